"""The C++ VUMPS driver (include/imps_vumps.hpp, run by tests/native/cpp_vumps_check.cpp) against
the Python driver (vumps.VumpsGPU) from the same state: both issue the same C-ABI calls in the
same order, so the energies, gradient norms and precisions of every sweep agree to the rounding
level (1e-12)."""
import subprocess

import numpy as np
import pytest

from imps_cpp_tools_gb300 import models
from imps_cpp_tools_gb300.vumps import VumpsGPU
from oracle import imps_oracle as O
from tests.test_gpu_parity import dev
from tests.test_gpu_vumps import B0, B1
from tests.test_native_host import _build_cpp_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("concurrent", [1, 0])
def test_cpp_vumps_matches_python_driver(cuda_ctx, tmp_path, concurrent):
    """concurrent = 1: the C++ driver's H_C eigensolves run on their own contexts and threads
    beside the H_AC eigensolve; 0: after it, on one stream."""
    d, I2K, h = models.build_model("xxz", J=1.0, Delta=-1.0)
    hnnz = models.h_nonzeros(h)
    dimvec = [B0, B1]
    AL, AR, C = O.randMPS_LR(2, I2K, dimvec, np.random.default_rng(7))
    flat = [O.mps_vec(AL[0]), O.mps_vec(AL[1]), O.mps_vec(AR[0]), O.mps_vec(AR[1]), O.bd_vec(C[1]), O.bd_vec(C[0])]
    nsweeps, tol, invetol = 3, 1e-12, 1e-12
    lines = [f"{d} {len(I2K[0])}", " ".join(str(x) for q in I2K for x in q)]
    for b in range(2):
        lines.append(str(len(dimvec[b])))
        lines += [" ".join(str(x) for x in q) + f" {m}" for q, m in sorted(dimvec[b].items())]
    lines.append(str(len(hnnz)))
    lines += [f"{r} {c} {v!r}" for (r, c, v) in hnnz]
    lines.append(f"{nsweeps} {tol!r} {invetol!r} 0.1 0 {concurrent}")
    lines += [" ".join(repr(float(x)) for x in v) for v in flat]
    inp = tmp_path / "vumps_input.txt"
    inp.write_text("\n".join(lines) + "\n")
    exe = _build_cpp_host(tmp_path, "cpp_vumps_check")
    r = subprocess.run([str(exe), str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "cpp vumps check ok" in r.stdout
    got = [list(map(float, ln.split()[2:])) for ln in r.stdout.splitlines() if ln.startswith("sweep ")]
    init = {"AL": [dev(flat[0]), dev(flat[1])], "AR": [dev(flat[2]), dev(flat[3])], "C": [dev(flat[4]), dev(flat[5])]}
    gpu = VumpsGPU(cuda_ctx, "xxz", dimvec=dimvec, init_state=init, fixed_tol=tol, InvETol=invetol, J=1.0, Delta=-1.0)
    assert len(got) == nsweeps
    for s in range(nsweeps):
        E, F, prec = gpu.sweep()
        e_cpp, f_cpp, p_cpp = np.array(got[s][0:2]), np.array(got[s][2:4]), np.array(got[s][4:6])  # then ms, applies
        assert np.abs(e_cpp - E).max() < 1e-12, (s, e_cpp, E)
        assert np.allclose(f_cpp, F, rtol=1e-9, atol=1e-14), (s, f_cpp, F)
        assert np.allclose(p_cpp, prec, rtol=1e-9, atol=1e-14), (s, p_cpp, prec)
