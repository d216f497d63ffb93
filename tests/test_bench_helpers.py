"""bench.py's host-side helpers on CPU: the committed ncu summary parses into
the roofline fields, and absent summaries give empty results, not errors."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_committed_summary_parses(bench):
    s = bench.ncu_summary("k_bu", 26)
    assert {"dram_bytes_per_launch", "ncu_mean_us", "search_dram_gbs_ncu"} <= set(s)
    assert bench.ncu_traffic("k_bu", 26) == s["dram_bytes_per_launch"] > 0
    m = bench.dram_measured("k_bu", 26, 6786.9)
    gbs = s["dram_bytes_per_launch"] / (s["ncu_mean_us"] * 1e-6) / 1e9
    assert m["kernel_gbs"] == pytest.approx(gbs)
    assert m["kernel_frac"] == pytest.approx(gbs / 6786.9)
    assert m["search_frac"] == pytest.approx(s["search_dram_gbs_ncu"] / 6786.9)
    # a measured fraction far above 1 would mean the summary is not the kernel's
    assert 0 < m["kernel_frac"] < 1.2 and 0 < m["search_frac"] < 1.2


def test_bytes_per_edge_view(bench):
    s = bench.ncu_summary("k_bu", 26)
    m = bench.dram_measured("k_bu", 26, 6786.9, 640.0, 1.07e9)
    bpe = s["search_dram_bytes_per_search"] / 1.07e9
    assert m["bytes_per_teps_edge"] == pytest.approx(bpe)
    assert m["at_value_gbs"] == pytest.approx(bpe * 640.0)
    assert m["at_value_frac_of_8tbs"] == pytest.approx(bpe * 640.0 / 8000.0)
    assert "at_value_gbs" not in bench.dram_measured("k_bu", 26, 6786.9)


def test_capture_settings(bench):
    cap = bench.ncu_summary("k_bu", 26)["settings"]
    assert set(cap) == {"alpha", "beta", "tile_edges", "bu_serial"}
    same = bench.capture_settings("k_bu", 26, cap["alpha"], cap["beta"],
                                  {"tile_edges": int(cap["tile_edges"]), "bu_serial": int(cap["bu_serial"])})
    assert same["match"]
    other = bench.capture_settings("k_bu", 26, cap["alpha"] * 2, cap["beta"], {})
    assert not other["match"] and other["run"]["tile_edges"] == 256


def test_missing_summary(bench):
    assert bench.ncu_summary("k_bu", 99) == {}
    assert bench.ncu_traffic("k_bu", 99) is None
    assert bench.dram_measured("k_bu", 99, 6786.9) is None


def test_size_flags_parse(bench, monkeypatch):
    monkeypatch.setattr("sys.argv", ["bench.py", "--tile-edges", "128", "--bu-serial", "8", "--alpha", "14"])
    a = bench.parse()
    assert (a.tile_edges, a.bu_serial, a.alpha, a.beta) == (128, 8, 14.0, None)
    assert (a.scale, a.roots, a.gpus) == (26, 64, 1)


def _profile_commands():
    """Every `python bench.py ...` command quoted in profiles/ (continuation
    lines joined), as argument lists."""
    import glob
    import shlex
    cmds = []
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*"))):
        text = open(path).read().replace("\\\n", " ")
        for line in text.splitlines():
            if "python bench.py" in line:
                args = shlex.split(line.split("python bench.py", 1)[1])
                cmds.append((os.path.basename(path), args))
    return cmds


def test_profile_commands_parse(bench, monkeypatch):
    """The captures under profiles/ can be re-run: their bench.py command
    lines use options the current bench.py accepts."""
    cmds = _profile_commands()
    assert cmds, "no bench.py command quoted under profiles/"
    for name, args in cmds:
        monkeypatch.setattr("sys.argv", ["bench.py"] + args)
        bench.parse()  # argparse exits on an unknown option
