"""CPU-side checks of the native library: it builds for sm_103a, exports
every entry point include/pa_gpu.h declares, refuses to run without a GPU
(no CPU fallback), and its input generators reproduce the reference's recipe.
No compute call runs here."""
import ctypes
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def native():
    from parallelalgorithms_gb300 import build as pabuild
    path = pabuild.build()
    return ctypes.CDLL(str(path))


def declared_entry_points() -> list[str]:
    names = []
    for h in (ROOT / "include").glob("*.h"):
        names += re.findall(r"^\s*(?:int|const char\*)\s+(pa_\w+)\s*\(", h.read_text(), re.M)
    return sorted(set(names))


def test_every_declared_entry_point_is_exported(native):
    names = declared_entry_points()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from parallelalgorithms_gb300 import _native
    declared = set(declared_entry_points())
    bound = set(_native.SIGNATURES) | {"pa_status_string", "pa_last_error_message"}
    assert declared <= bound, declared - bound


def test_built_for_sm103a_only(native):
    # the fatbin of an sm_103a-only build names that architecture; the
    # build command pins the single -gencode
    from parallelalgorithms_gb300 import build as pabuild
    assert pabuild.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_no_gpu_means_loud_failure(native):
    import parallelalgorithms_gb300 as pa
    if pa.lib().pa_device_available():
        pytest.skip("a GPU is present")
    a = np.arange(1000, dtype=np.uint32)[::-1].copy()
    with pytest.raises(pa.PaError) as e:
        pa.SortRadixPar(a, None, a.size)
    assert e.value.status == 5  # PA_ERR_NO_DEVICE
    np.testing.assert_array_equal(a, np.arange(1000, dtype=np.uint32)[::-1])  # untouched: no CPU fallback
    with pytest.raises(pa.PaError):
        pa.SumParallelNonRecursive(a, 0, a.size)


def test_argument_errors_are_reported_before_any_device_work(native):
    import parallelalgorithms_gb300 as pa
    lib = pa.lib()
    out = np.zeros(1, np.uint32)
    a = np.zeros(4, np.uint32)
    # k out of range
    rc = lib.pa_select_u32(ctypes.c_void_p(a.ctypes.data), 4, 4, ctypes.c_void_p(out.ctypes.data), None)
    assert rc == 1
    # shift out of range
    h = np.zeros(256, np.uint64)
    rc = lib.pa_hist_one_byte_u32(ctypes.c_void_p(a.ctypes.data), 4, 32, ctypes.c_void_p(h.ctypes.data), None)
    assert rc == 1
    assert b"shift" in lib.pa_last_error_message()
    # zero-length sort is a no-op success
    assert lib.pa_sort_u32(None, None, 0, None) == 0


def test_generators_reproduce_the_reference_recipe(golden):
    from parallelalgorithms_gb300 import workloads
    np.testing.assert_array_equal(workloads.uniform_u32(8191, seed=1234), golden["in_uniform_8191"])
    a = workloads.uniform_u32(1000, seed=99)
    b = workloads.uniform_u32(1000, seed=99)
    np.testing.assert_array_equal(a, b)
    f = workloads.normal_specials_f32(200000)
    bits = f.view(np.uint32)
    for special in (0x0, 0x80000000, 0x7F800000, 0xFF800000):
        frac = np.mean(bits == special)
        assert 0.007 < frac < 0.013, (hex(special), frac)
    den = ((bits & 0x7F800000) == 0) & ((bits & 0x7FFFFF) != 0)
    assert 0.007 < den.mean() < 0.013
    z = workloads.zipf_u64(100000)
    vals, counts = np.unique(z, return_counts=True)
    assert counts.max() > 5000 and vals.size > 1000
    s = workloads.log_uniform_sizes(4096, 1e3, 4e6)
    assert s.min() >= 1000 and s.max() <= 4_000_000


def test_dropin_headers_compile_and_link(native, tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "dropin"
    r = subprocess.run([gxx, "-std=c++17", "-O1", f"-I{ROOT / 'include' / 'ParallelAlgorithms'}",
                        f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "dropin_main.cpp"),
                        f"-L{ROOT / 'parallelalgorithms_gb300'}", "-lpa_gb300", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
