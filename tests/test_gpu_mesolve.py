"""GPU mesolve (Vern7 on the device) against the reference's own mesolve results.

Tolerances: complex128 results must agree with the reference within
atol 1e-8 / rtol 1e-6 on expectation values; the mixed (complex64 stages, FP64
state and control) and single forms state their error against the FP64 result.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, csr_from, golden

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ATOL, RTOL = 1e-8, 1e-6


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _close(got, want, atol=ATOL, rtol=RTOL):
    got, want = np.asarray(got), np.asarray(want)
    assert np.all(np.abs(got - want) <= atol + rtol * np.abs(want)), np.abs(got - want).max()


def test_jc_mesolve_double_matches_reference():
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import solve_system
    g = golden("jc_mesolve.npz")
    s = S.jaynes_cummings()
    res = solve_system(s, g["tlist"], {"store_final_state": True})
    for k in range(2):
        _close(res.expect[k].real, g["expect"][k])
    _close(res.final_state, g["final"], atol=1e-8)
    assert res.stats["steps"] >= len(g["step_ends"])


def test_jc_step_sequence_is_the_reference():
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.vern7 import GpuVern7
    g = golden("jc_mesolve.npz")
    s = S.jaynes_cummings()
    ig = GpuVern7(DeviceOperator(s.terms))
    ig.set_initial_value(torch.from_numpy(g["rho0"]).cuda(), 0.0)
    ends = []
    while ig.t_front < 20.0:
        ig.integrate(20.0, step=True)
        ig.check()
        ends.append(ig.t_front)
    assert len(ends) == len(g["step_ends"])
    np.testing.assert_allclose(ends, g["step_ends"], rtol=1e-8)


def test_jc_mixed_step_sequence_follows_the_reference():
    """The mixed form keeps the step-size control in FP64: the error estimate is summed
    in float-float from the complex64 stage vectors and the WRMS norm and step factor
    are FP64.  It takes the reference's steps one for one (same count, same accept /
    reject sequence).  The step ends still move: the error estimate is a small
    difference of stage vectors (sum_j e_j k_j, a few 1e-7 of |k| at these tolerances),
    so the 6e-8 rounding of each complex64 k_j shifts err by percents and the next step,
    through err^(-1/8), by a fraction of that -- measured 5e-3 here, bounded at 2e-2."""
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.vern7 import GpuVern7
    g = golden("jc_mesolve.npz")
    s = S.jaynes_cummings()
    ig = GpuVern7(DeviceOperator(s.terms, dtype="c64"), precision="mixed")
    ig.set_initial_value(torch.from_numpy(g["rho0"]).cuda(), 0.0)
    ends = []
    while ig.t_front < 20.0:
        ig.integrate(20.0, step=True)
        ig.check()
        ends.append(ig.t_front)
    rel = np.max(np.abs(np.asarray(ends) - g["step_ends"]) / g["step_ends"])
    print(f"\nmixed step ends vs the reference: {len(ends)} steps, max rel diff {rel:.2e}")
    assert len(ends) == len(g["step_ends"])
    assert rel <= 2e-2


@pytest.mark.parametrize("L", [3, 4])
def test_ising_td_mesolve_double_matches_reference(L):
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import solve_system
    g = golden(f"ising_L{L}_mesolve.npz")
    s = S.ising_chain(L)
    res = solve_system(s, g["tlist"], {"store_final_state": True})
    for k in range(L):
        _close(res.expect[k].real, g["expect"][k])
    _close(res.final_state, g["final"])


@pytest.mark.parametrize("prec,bound", [("mixed", 2e-6), ("single", 2e-5)])
def test_ising_reduced_precision_error_vs_fp64(prec, bound):
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import solve_system
    g = golden("ising_L4_mesolve.npz")
    s = S.ising_chain(4)
    res = solve_system(s, g["tlist"], {"precision": prec})
    err = max(np.abs(res.expect[k].real - g["expect"][k]).max() for k in range(4))
    print(f"\n{prec}: max |<sz_i> - FP64 reference| = {err:.3e}")
    assert err < bound


def test_too_much_work_raises_like_reference():
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import solve_system
    from qutip_gb300.vern7 import IntegratorError
    s = S.jaynes_cummings()
    with pytest.raises(IntegratorError, match="Too much work"):
        solve_system(s, np.linspace(0, 20, 3), {"nsteps": 2})


def test_mesolve_api_with_string_coefficient():
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import mesolve
    from oracle.solvers import mesolve as omesolve
    L = 3
    s = S.ising_chain(L)
    (h0, _), (h1, _) = s.h_terms
    tl = np.linspace(0, 2, 11)
    psi0 = np.zeros(2 ** L)
    psi0[0] = 1
    res = mesolve([h0, [h1, "cos(w*t)"]], psi0, tl, s.c_ops, s.e_ops, args={"w": 1.3})
    want, _ = omesolve(s.terms, s.state0, tl, s.e_ops)
    for k in range(L):
        _close(res.expect[k], want[k])


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "ising_L10_expect.npz")),
                    reason="full-size golden not generated")
def test_ising_L10_full_size_matches_reference():
    from qutip_gb300 import systems as S
    from qutip_gb300.solver import solve_system
    g = golden("ising_L10_expect.npz")
    s = S.ising_chain(10)
    res = solve_system(s, g["tlist"])
    for k in range(10):
        _close(res.expect[k].real, g["expect"][k])
    resm = solve_system(s, g["tlist"], {"precision": "mixed"})
    err = max(np.abs(resm.expect[k].real - g["expect"][k]).max() for k in range(10))
    print(f"\nIsing L=10 mixed: max |<sz_i> - FP64 reference| = {err:.3e}")
    assert err < 1e-5


def test_ising_L12_mixed_against_complex128_gpu():
    """Config 5 at full size: the L = 12 chain (Liouvillian 16,777,216 rows, 469,762,047
    entries assembled on the device), tlist linspace(0, 5, 51).  The mixed form (complex64
    matvec and stages, FP64 state, step control and expectation values) against the
    complex128 solve of the same generator: relative error of every sigma_z trajectory
    (max_t |diff| / max_t |want|) at most 1e-6, the stated bound of the mixed form."""
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import DeviceOperator
    from qutip_gb300.solver import ExpectOps, solve_system
    from qutip_gb300.superop import liouvillian_groups
    s = S.ising_chain(12, build_terms=False)
    groups = liouvillian_groups(s.h_terms, s.c_ops)
    op64 = DeviceOperator.from_device_groups(groups, "c64")
    op128 = DeviceOperator.from_device_groups(groups, "c128")
    del groups
    torch.cuda.empty_cache()
    assert op64.n_rows == 4 ** 12 and op64.nnz == 469762047
    ex = ExpectOps(s.e_ops)
    tl = np.linspace(0.0, 5.0, 51)
    r128 = solve_system(s, tl, {"precision": "double"}, op=op128, ex=ex)
    r64 = solve_system(s, tl, {"precision": "mixed"}, op=op64, ex=ex)
    rel = max(float(np.max(np.abs(a.real - b.real)) / np.max(np.abs(b.real)))
              for a, b in zip(r64.expect, r128.expect))
    print(f"\nIsing L=12 mixed vs complex128 GPU: max relative error {rel:.2e}, "
          f"{r64.stats['steps']} / {r128.stats['steps']} steps")
    assert r64.stats["steps"] == r128.stats["steps"]
    assert rel <= 1e-6
    del op64, op128
    torch.cuda.empty_cache()
