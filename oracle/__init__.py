"""CPU oracle for the QuTiP time-evolution hot path.

TEST INFRASTRUCTURE ONLY.  This package restates, in numpy/scipy FP64, the
reference algorithms that ``qutip_gb300`` replaces on the GPU: the CSR/Dia
matvec kernels, the expect/wrmn reductions, the Verner-7 explicit Runge-Kutta
integrator with dense output and the Monte-Carlo jump integrator.  It is used
only by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg, always as the checker and never as the measured or shipped path.

Pinning: every restatement here is checked against golden vectors produced by
the reference QuTiP itself (built from source by ``oracle/build_ref.py``) and
committed under ``tests/golden/`` together with the script that made them.
"""
