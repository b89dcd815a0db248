"""A C++ caller written against the reference's headers
(tests/cpp/dropin_main.cpp) is compiled against include/ParallelAlgorithms/
and linked to libpa_gb300.so, then run on the GPU; it checks every result
against the C++ standard library (std::stable_sort, std::nth_element,
std::accumulate) the way the reference's benchmarks do."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("n", [7, 100, 1_000_003, 10_000_000])
def test_dropin_cpp_caller(pa, tmp_path, n):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.fail("g++ is required to build the C++ caller")
    exe = tmp_path / "dropin"
    lib_dir = ROOT / "parallelalgorithms_gb300"
    r = subprocess.run([gxx, "-std=c++17", "-O2", f"-I{ROOT / 'include' / 'ParallelAlgorithms'}",
                        f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "dropin_main.cpp"),
                        f"-L{lib_dir}", "-lpa_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe), str(n)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert f"OK n={n}" in run.stdout
