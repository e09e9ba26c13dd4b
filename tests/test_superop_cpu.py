"""Device Liouvillian assembly (run here on CPU tensors): the same generator as the
host construction, the same coefficient groups, and the same sliced-ELLPACK
layout as the host layout builder."""
import numpy as np
import pytest
import scipy.sparse as sp

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("L", [3, 5])
def test_liouvillian_groups_match_host_construction(L):
    from qutip_gb300 import systems as S
    from qutip_gb300.superop import liouvillian_groups
    s = S.ising_chain(L)
    groups = liouvillian_groups(s.h_terms, s.c_ops, device="cpu")
    assert len(groups) == len(s.terms)
    n = s.dim * s.dim
    for (indptr, indices, data, coeff), (m, c_host) in zip(groups, s.terms):
        got = sp.csr_matrix((data.numpy(), indices.numpy(), indptr.numpy()), shape=(n, n))
        assert (coeff is None) == (c_host is None)
        if coeff is not None:
            assert coeff.key() == c_host.key()
        diff = abs(got - sp.csr_matrix(m)).max()
        assert diff <= 1e-14 * max(1.0, abs(sp.csr_matrix(m)).max())


def test_device_sliced_layout_matches_host_layout():
    from qutip_gb300 import systems as S
    from qutip_gb300.operator import sliced_layout
    from qutip_gb300.superop import device_sliced_layout
    s = S.ising_chain(5)
    n = s.dim * s.dim
    rp, w, col, val, total = sliced_layout([m for m, _ in s.terms], n)
    groups = []
    for m, c in s.terms:
        m = sp.csr_matrix(m)
        m.sort_indices()
        groups.append((torch.from_numpy(m.indptr.astype(np.int64)),
                       torch.from_numpy(m.indices.astype(np.int64)),
                       torch.from_numpy(m.data.astype(np.complex128)), c))
    rp2, w2, col2, val2, total2 = device_sliced_layout(groups, n)
    assert total2 == total
    np.testing.assert_array_equal(rp2.numpy(), rp)
    np.testing.assert_array_equal(w2.numpy(), w)
    np.testing.assert_array_equal(col2.numpy(), col)
    np.testing.assert_array_equal(val2.numpy(), val)


def test_jaynes_cummings_groups():
    from qutip_gb300 import systems as S
    from qutip_gb300.superop import liouvillian_groups
    s = S.jaynes_cummings(7, kind="me")
    groups = liouvillian_groups(s.h_terms, s.c_ops, device="cpu")
    n = s.dim * s.dim
    got = sum(sp.csr_matrix((d.numpy(), i.numpy(), p.numpy()), shape=(n, n)) for p, i, d, _ in groups)
    want = sum(sp.csr_matrix(m) for m, _ in s.terms)
    assert abs(got - want).max() <= 1e-13
