"""CPU oracle for the IMPS block-sparse hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference arm may import this package, and only as the checker (or as the
timed reference-CPU restatement).  The product path in
``imps_cpp_tools_gb300`` never imports it; the product fails loudly when its
CUDA library is missing.

Parity status: UNPINNED by the reference.  The reference (IMPS_CPP_tools,
C++ over armadillo/ARPACK/LAPACK) ships no tests, golden vectors or fixtures,
and it cannot be compiled here (armadillo, ARPACK and a Fortran runtime are
absent).  The oracle is instead pinned by mathematics: dense (symmetry-free)
re-evaluation of every block-sparse contraction, the reference's own inline
identities (gauge, isometry, InvertE fixed-point identity), and exact or
perturbative physics of the reference's models:
* the Bethe-ansatz ground-state energy of the Heisenberg chain;
* the exact transverse-field Ising energy and quasiparticle dispersion, with Z(2) charges;
* strong-coupling perturbation theory of the Bose-Hubbard and Potts chains;
* total charge on the excitation space equal to the sector's charge shift times the identity.
"""
