"""Generate the warmed VUMPS states the benchmark starts its timed sweeps from (GPU).

    python tests/golden/make_warm_states.py [--out DIR] [--workload NAME ...]

For each workload: the GPU driver (VumpsGPU, FP64) from randMPS_LR with seed 1, run with the
reference's tolerance schedule tol = min(max(prec/100, 1e-12), 1e-6) (VUMPS_main.cpp:177) for
a fixed number of sweeps, so that the state is past the chaotic first sweeps of a random start
and the timed sweeps at the fixed tolerance 1e-12 start where both the GPU path and the CPU
restatement converge in bounded work.  Saved: the flat AL(n), AR(n), C[b] buffers in the
reference's Vectorize order (C[b] is the centre matrix on bond b), the sweeps run, the energy
and the gradient norm.  The device kernels reduce in a fixed order, so a rerun on a GB300
reproduces the file.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

def main():
    import torch
    from imps_cpp_tools_gb300 import blocks as B
    from imps_cpp_tools_gb300 import workload as W
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--workload", nargs="*", default=sorted(W.WARM_SWEEPS))
    args = ap.parse_args()
    ctx = B.Context(0)
    ctx.set_stream(torch.cuda.current_stream())
    for name in args.workload:
        h, E, F = W.warm_on_device(ctx, name, verbose=True)
        out = {f"{k}{n}": h[k][n] for k in ("AL", "AR", "C") for n in range(2)}
        out.update(sweeps=W.WARM_SWEEPS[name], energy=E, grad_norm=F, seed=W.WARM_SEED)
        path = os.path.join(args.out, f"warm_{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{name}: {W.WARM_SWEEPS[name]} sweeps, E={E.mean():.12f} |grad|={F.max():.2e} -> {path}", flush=True)


if __name__ == "__main__":
    main()
