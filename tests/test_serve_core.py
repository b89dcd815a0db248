"""The serving loop's scheduling policy (admission by HBM budget, coalescing
of 32-bit sorts, in-flight cap, FIFO, thread-safe submission) exercised on
the CPU through a fake device backend: tests/cpp/serve_core_test.cpp."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_serve_core_policy_with_fake_backend(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "serve_core_test"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-pthread", f"-I{ROOT / 'parallelalgorithms_gb300' / 'csrc'}",
                        str(ROOT / "tests" / "cpp" / "serve_core_test.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "OK" in run.stdout
