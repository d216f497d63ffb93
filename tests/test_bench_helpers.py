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
    s = bench.ncu_summary("k_bu_kinds", 26)
    assert {"first_dram_bytes_per_launch", "list_dram_bytes_per_launch",
            "first_ncu_us_scale24", "first_dram_bytes_scale24"} <= set(s)
    # the scale-26 traffic is the scale-24 capture times 4
    assert s["first_dram_bytes_per_launch"] == pytest.approx(4 * s["first_dram_bytes_scale24"])
    assert s["list_dram_bytes_per_launch"] == pytest.approx(4 * s["list_dram_bytes_scale24"])
    assert bench.kind_traffic("bu_first", 26) == s["first_dram_bytes_per_launch"] > 0
    assert bench.kind_traffic("td", 26) is None
    m = bench.dram_measured(26, 6786.9)
    gbs = s["first_dram_bytes_scale24"] / (s["first_ncu_us_scale24"] * 1e-6) / 1e9
    assert m["bu_first"]["gbs"] == pytest.approx(gbs)
    assert m["bu_first"]["frac"] == pytest.approx(gbs / 6786.9)
    # a measured fraction far above 1 would mean the summary is not the kernel's
    for kind in ("bu_first", "bu_list"):
        assert 0 < m[kind]["frac"] < 1.2


def test_capture_settings(bench):
    cap = bench.ncu_summary("k_bu_kinds", 26)["settings"]
    assert set(cap) == {"alpha", "beta", "tile_edges", "bu_serial"}
    same = bench.capture_settings("k_bu_kinds", 26, cap["alpha"], cap["beta"],
                                  {"tile_edges": int(cap["tile_edges"]), "bu_serial": int(cap["bu_serial"])})
    assert same["match"]
    other = bench.capture_settings("k_bu_kinds", 26, cap["alpha"] * 2, cap["beta"], {})
    assert not other["match"] and other["run"]["tile_edges"] == 256


def test_missing_summary(bench):
    assert bench.ncu_summary("k_bu_kinds", 99) == {}
    assert bench.kind_traffic("bu_first", 99) is None
    assert bench.dram_measured(99, 6786.9) is None
    assert bench.capture_settings("k_bu_kinds", 99, 25, 1000, {}) is None


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
