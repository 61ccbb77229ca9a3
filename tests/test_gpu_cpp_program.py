"""The C++ grouped-GEMM program builder (include/imps_gb300.hpp, tests/native/cpp_program_check.cpp)
run on the device against the same products on the host."""
import subprocess

import pytest

from tests.test_native_host import _build_cpp_host

pytestmark = pytest.mark.gpu


def test_cpp_program_runs(tmp_path):
    exe = _build_cpp_host(tmp_path, "cpp_program_check")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "cpp program check ok" in r.stdout
