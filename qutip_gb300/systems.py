"""Operator builders for the open-system workloads this package is measured on.

Everything here is host-side scipy code that runs once per system, off the hot
loop.  The conventions are QuTiP's, so that a Liouvillian built here acts on the
same column-stacked density-matrix vector as the reference's:

* ``tensor`` is the Kronecker product with the first factor most significant
  (qutip/core/tensor.py);
* ``destroy(N)`` has ``sqrt(n)`` on the first super-diagonal, ``sigmaz`` is
  ``diag(1, -1)``, ``sigmam = |1><0|`` and ``basis(2, 0)`` is the excited
  ("up", sigma_z = +1) state (qutip/core/operators.py, qutip/core/states.py);
* vec(rho) stacks columns, so ``spre(A) = I (x) A`` and ``spost(A) = A^T (x) I``
  (qutip/core/superoperator.py:291-334);
* ``lindblad_dissipator(c) = spre(c) spost(c^+) - 1/2 spre(c^+c) - 1/2 spost(c^+c)``
  (qutip/core/superoperator.py:161-229) and the Liouvillian of a Hamiltonian is
  ``-i (spre(H) - spost(H))`` (qutip/core/superoperator.py:116-134).

A time-dependent generator is returned as a list of ``(csr_matrix, coefficient)``
terms, the shape ``QobjEvo.to_list()`` has (qutip/core/cy/qobjevo.pyx:869), where
the coefficient is ``None`` for the constant part or a
:class:`qutip_gb300.coefficients.Coefficient`.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

from .coefficients import Coefficient, coefficient

__all__ = [
    "destroy", "qeye", "sigmaz", "sigmax", "sigmam", "sigmap", "basis", "tensor",
    "spre", "spost", "lindblad_dissipator", "liouvillian", "OpenSystem",
    "jaynes_cummings", "ising_chain", "bose_hubbard_trimer", "merge_terms",
]


def _csr(a) -> sp.csr_matrix:
    m = sp.csr_matrix(a, dtype=np.complex128)
    m.sum_duplicates()
    m.eliminate_zeros()
    m.sort_indices()
    return m


def destroy(n: int) -> sp.csr_matrix:
    return _csr(sp.diags(np.sqrt(np.arange(1, n, dtype=np.float64)), 1, shape=(n, n)))


def qeye(n: int) -> sp.csr_matrix:
    return _csr(sp.identity(n))


def sigmaz() -> sp.csr_matrix:
    return _csr(np.array([[1, 0], [0, -1]]))


def sigmax() -> sp.csr_matrix:
    return _csr(np.array([[0, 1], [1, 0]]))


def sigmam() -> sp.csr_matrix:
    return _csr(np.array([[0, 0], [1, 0]]))


def sigmap() -> sp.csr_matrix:
    return _csr(np.array([[0, 1], [0, 0]]))


def basis(n: int, k: int) -> np.ndarray:
    v = np.zeros(n, dtype=np.complex128)
    v[k] = 1.0
    return v


def tensor(*ops):
    out = ops[0]
    for o in ops[1:]:
        if isinstance(out, np.ndarray) and out.ndim == 1:
            out = np.kron(out, o)
        else:
            out = sp.kron(out, o, format="csr")
    return out if isinstance(out, np.ndarray) else _csr(out)


def spre(a) -> sp.csr_matrix:
    return _csr(sp.kron(sp.identity(a.shape[0]), a, format="csr"))


def spost(a) -> sp.csr_matrix:
    return _csr(sp.kron(a.T, sp.identity(a.shape[0]), format="csr"))


def lindblad_dissipator(c) -> sp.csr_matrix:
    c = _csr(c)
    cd = _csr(c.conj().T)
    cdc = _csr(cd @ c)
    return _csr(spre(c) @ spost(cd) - 0.5 * spre(cdc) - 0.5 * spost(cdc))


def liouvillian(h=None, c_ops=()) -> sp.csr_matrix:
    n = (h if h is not None else c_ops[0]).shape[0]
    out = sp.csr_matrix((n * n, n * n), dtype=np.complex128)
    if h is not None:
        out = out + (-1j) * (spre(h) - spost(h))
    for c in c_ops:
        out = out + lindblad_dissipator(c)
    return _csr(out)


def merge_terms(terms):
    """Sum terms that share a coefficient (``None`` = constant), keeping order.

    Mirrors ``QobjEvo.compress`` (qutip/core/cy/qobjevo.pyx:816): constant parts
    are merged into one operator and terms with an identical coefficient object
    are merged into one.
    """
    out: list[list] = []
    for op, coeff in terms:
        key = None if coeff is None else coeff.key()
        for item in out:
            ikey = None if item[1] is None else item[1].key()
            if ikey == key:
                item[0] = _csr(item[0] + op)
                break
        else:
            out.append([_csr(op), coeff])
    return [(op, c) for op, c in out]


@dataclass
class OpenSystem:
    """One workload: generator terms, collapse operators, initial state, e_ops.

    ``terms`` is the Liouvillian (``kind == "me"``) or the effective
    non-Hermitian ``-iH - 1/2 sum c^+c`` (``kind == "mc"``) as coefficient terms.
    ``state0`` is vec(rho0) (column-stacked) for ``"me"`` and the ket for
    ``"mc"``.  ``e_ops`` are Hilbert-space operators.
    """
    name: str
    kind: str
    dim: int
    terms: list
    state0: np.ndarray
    e_ops: list
    c_ops: list = field(default_factory=list)
    h_terms: list = field(default_factory=list)
    meta: dict = field(default_factory=dict)


def _me_terms(h_terms, c_ops):
    terms = []
    for h, coeff in h_terms:
        terms.append(((-1j) * (spre(h) - spost(h)), coeff))
    if c_ops:
        d = sum((lindblad_dissipator(c) for c in c_ops[1:]), lindblad_dissipator(c_ops[0]))
        terms.append((_csr(d), None))
    return merge_terms(terms)


def _mc_terms(h_terms, c_ops):
    terms = [((-1j) * h, coeff) for h, coeff in h_terms]
    for c in c_ops:
        cdc = _csr(c.conj().T @ c)
        terms.append((-0.5 * cdc, None))
    return merge_terms(terms)


def jaynes_cummings(n_cav=10, wc=2 * np.pi, wa=2 * np.pi, g=2 * np.pi * 0.05,
                    kappa=0.005, gamma=0.05, kind="me") -> OpenSystem:
    """Driven-damped Jaynes-Cummings: cavity cutoff ``n_cav`` (x) qubit.

    ``H = wc a^+a + wa sz/2 + g (a s+ + a^+ s-)``, collapse operators
    ``sqrt(kappa) a`` and ``sqrt(gamma) s-``; initial state ``|0> (x) |e>``;
    e_ops ``a^+a`` and ``sz``.
    """
    a = tensor(destroy(n_cav), qeye(2))
    sm = tensor(qeye(n_cav), sigmam())
    sz = tensor(qeye(n_cav), sigmaz())
    h = _csr(wc * (a.conj().T @ a) + wa * 0.5 * sz
             + g * (a @ sm.conj().T + a.conj().T @ sm))
    c_ops = [_csr(np.sqrt(kappa) * a), _csr(np.sqrt(gamma) * sm)]
    psi0 = tensor(basis(n_cav, 0), basis(2, 0))
    e_ops = [_csr(a.conj().T @ a), sz]
    d = 2 * n_cav
    if kind == "me":
        rho0 = np.outer(psi0, psi0.conj())
        return OpenSystem("jaynes_cummings", "me", d, _me_terms([(h, None)], c_ops),
                          rho0.reshape(-1, order="F").copy(), e_ops, c_ops, [(h, None)],
                          dict(n_cav=n_cav, wc=wc, wa=wa, g=g, kappa=kappa, gamma=gamma))
    return OpenSystem("jaynes_cummings", "mc", d, _mc_terms([(h, None)], c_ops), psi0,
                      e_ops, c_ops, [(h, None)],
                      dict(n_cav=n_cav, wc=wc, wa=wa, g=g, kappa=kappa, gamma=gamma))


def ising_chain(n_sites=10, J=1.0, h=None, omega=1.3, gamma_minus=0.05, gamma_z=0.02,
                seed=1234, kind="me", build_terms=True) -> OpenSystem:
    """Dissipative transverse-field Ising chain with an oscillating field.

    ``H(t) = -J sum_i sz_i sz_{i+1} - sum_i h_i cos(omega t) sx_i`` (open chain),
    ``h_i ~ U[0.5, 1.5]`` from ``numpy.random.default_rng(seed)``; collapse
    operators ``sqrt(gamma_minus) s-_i`` and ``sqrt(gamma_z) sz_i`` on every
    site; initial state all spins up; e_ops ``sz_i``.  With ``build_terms=False``
    the Liouvillian is left to :func:`qutip_gb300.superop.liouvillian_groups`
    (device assembly) and ``terms`` is ``None``.
    """
    if h is None:
        h = np.random.default_rng(seed).uniform(0.5, 1.5, n_sites)
    ops = lambda o, i: tensor(*[o if k == i else qeye(2) for k in range(n_sites)])  # noqa: E731
    sz = [ops(sigmaz(), i) for i in range(n_sites)]
    sx = [ops(sigmax(), i) for i in range(n_sites)]
    sm = [ops(sigmam(), i) for i in range(n_sites)]
    dim = 2 ** n_sites
    h0 = sp.csr_matrix((dim, dim), dtype=np.complex128)
    for i in range(n_sites - 1):
        h0 = h0 + (-J) * (sz[i] @ sz[i + 1])
    h1 = sp.csr_matrix((dim, dim), dtype=np.complex128)
    for i in range(n_sites):
        h1 = h1 + (-h[i]) * sx[i]
    h0, h1 = _csr(h0), _csr(h1)
    cos = coefficient("cos(w*t)", args={"w": omega})
    c_ops = [_csr(np.sqrt(gamma_minus) * s) for s in sm] + [_csr(np.sqrt(gamma_z) * s) for s in sz]
    psi0 = tensor(*[basis(2, 0) for _ in range(n_sites)])
    h_terms = [(h0, None), (h1, cos)]
    meta = dict(n_sites=n_sites, J=J, h=np.asarray(h), omega=omega, gamma_minus=gamma_minus,
                gamma_z=gamma_z, seed=seed)
    if kind == "me":
        rho0 = np.zeros(dim * dim, dtype=np.complex128)
        i0 = int(np.flatnonzero(psi0)[0])
        rho0[i0 + dim * i0] = 1.0
        terms = _me_terms(h_terms, c_ops) if build_terms else None
        return OpenSystem("ising_chain", "me", dim, terms, rho0, sz, c_ops, h_terms, meta)
    return OpenSystem("ising_chain", "mc", dim, _mc_terms(h_terms, c_ops), psi0, sz, c_ops,
                      h_terms, meta)


def bose_hubbard_trimer(cutoff=8, J=1.0, U=0.5, F=0.3, kappa=0.1, topology="ring",
                        kind="mc") -> OpenSystem:
    """Dissipative Bose-Hubbard trimer: three sites with ``cutoff`` levels each.

    ``H = -J sum_<ij> (a_i^+ a_j + h.c.) + U/2 sum_i n_i (n_i - 1) + F (a_0 + a_0^+)``
    with nearest-neighbour pairs of a ring (0-1, 1-2, 2-0) or a chain; collapse
    operators ``sqrt(kappa) a_i``; initial state vacuum; e_ops ``n_i``.
    """
    a = [tensor(*[destroy(cutoff) if k == i else qeye(cutoff) for k in range(3)])
         for i in range(3)]
    n = [_csr(x.conj().T @ x) for x in a]
    pairs = [(0, 1), (1, 2), (2, 0)] if topology == "ring" else [(0, 1), (1, 2)]
    dim = cutoff ** 3
    h = sp.csr_matrix((dim, dim), dtype=np.complex128)
    for i, j in pairs:
        h = h + (-J) * (a[i].conj().T @ a[j] + a[j].conj().T @ a[i])
    for i in range(3):
        h = h + (U / 2) * (n[i] @ (n[i] - sp.identity(dim)))
    h = _csr(h + F * (a[0] + a[0].conj().T))
    c_ops = [_csr(np.sqrt(kappa) * x) for x in a]
    psi0 = basis(dim, 0)
    meta = dict(cutoff=cutoff, J=J, U=U, F=F, kappa=kappa, topology=topology)
    if kind == "mc":
        return OpenSystem("bose_hubbard_trimer", "mc", dim, _mc_terms([(h, None)], c_ops), psi0,
                          n, c_ops, [(h, None)], meta)
    rho0 = np.zeros(dim * dim, dtype=np.complex128)
    rho0[0] = 1.0
    return OpenSystem("bose_hubbard_trimer", "me", dim, _me_terms([(h, None)], c_ops), rho0, n,
                      c_ops, [(h, None)], meta)
