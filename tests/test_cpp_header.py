"""include/g5bfs.hpp, the C++ host classes over the C ABI, compiles against
the in-tree library and behaves on the host (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_header_builds_and_runs(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    import gpugraph500_gb300 as g5
    if not os.path.exists(g5.LIB_PATH):
        from gpugraph500_gb300 import build
        build.build()
    libdir = os.path.dirname(g5.LIB_PATH)
    exe = str(tmp_path / "g5bfs_hpp_check")
    subprocess.run([gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "g5bfs_hpp_check.cpp"), "-L", libdir, "-lg5bfs",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "g5bfs.hpp ok" in r.stdout


@pytest.mark.gpu
def test_cpp_classes_on_gpu_match_oracle(tmp_path):
    """g5::CudaBFS, g5::Batch and g5::Server from C++: parents equal the
    oracle's (the device validator accepts the plain ones); g5::GpuSimd
    round-trips a compressed queue."""
    import numpy as np

    import oracle as orc
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    import gpugraph500_gb300 as g5
    libdir = os.path.dirname(g5.LIB_PATH)
    exe = str(tmp_path / "g5bfs_hpp_gpu")
    subprocess.run([gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "g5bfs_hpp_gpu.cpp"), "-L", libdir, "-lg5bfs",
                    "-I", "/usr/local/cuda/include", "-L", "/usr/local/cuda/lib64", "-lcudart",
                    "-Wl,-rpath," + libdir, "-Wl,-rpath,/usr/local/cuda/lib64", "-o", exe], check=True)
    scale = 12
    ro, col = orc.build_csr(1 << scale, orc.kronecker(scale))
    roots = [int(r) for r in orc.select_roots(ro, 3)]
    out = str(tmp_path / "parents.bin")
    r = subprocess.run([exe, str(scale), out] + [str(x) for x in roots], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    n, k = 1 << scale, len(roots)
    raw = open(out, "rb").read()
    assert len(raw) == 8 * n * k + 4 * n * k + 8 * n * k
    plain = np.frombuffer(raw[: 8 * n * k], np.int64).reshape(k, n)
    batch = np.frombuffer(raw[8 * n * k: 12 * n * k], np.uint32).reshape(n, k)
    served = np.frombuffer(raw[12 * n * k:], np.int64).reshape(k, n)
    for i, root in enumerate(roots):
        want = orc.bfs(ro, col, root)[0]
        assert np.array_equal(plain[i], want), root
        assert np.array_equal(batch[:, i].astype(np.int64), np.where(want < 0, 0xFFFFFFFF, want)), root
        assert np.array_equal(served[i], want), root
