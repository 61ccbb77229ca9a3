"""The C++ host program over the C ABI (tests/native/cpp_host_check.cpp, include/imps_gb300.hpp)
run on the device: left isometry, TMDominantEig, eigs_n and InvertE_proj through the
reference-named functors."""
import subprocess

import pytest

from tests.test_native_host import _build_cpp_host

pytestmark = pytest.mark.gpu


def test_cpp_host_program_runs(tmp_path):
    exe = _build_cpp_host(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "cpp host check ok" in r.stdout
