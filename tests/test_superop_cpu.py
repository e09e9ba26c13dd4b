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


def _split_terms(L):
    """The Ising Liouvillian as separate terms, two of them sharing the constant group and
    two sharing one coefficient, so that merging has to sum overlapping entries."""
    from qutip_gb300 import systems as S
    s = S.ising_chain(L)
    (m0, c0), (m1, c1) = s.terms[0], s.terms[1]
    m0 = sp.csr_matrix(m0)
    half = sp.csr_matrix(m0.multiply(sp.random(m0.shape[0], m0.shape[1], density=0.3,
                                               random_state=3, format="csr") != 0))
    rest = sp.csr_matrix(m0 - half)
    m1 = sp.csr_matrix(m1)
    return [(rest, None), (m1 * 0.25, c1), (half, None), (m1 * 0.75, c1), (sp.diags(m0.diagonal()).tocsr(), None)]


def test_device_term_groups_equal_the_host_merge_bit_for_bit():
    from qutip_gb300.superop import device_term_groups
    from qutip_gb300.systems import merge_terms
    terms = _split_terms(4)
    host = merge_terms(terms)
    dev = device_term_groups(terms, device="cpu")
    assert len(dev) == len(host)
    n = terms[0][0].shape[0]
    for (ip, ix, v, c), (m, ch) in zip(dev, host):
        assert (c is None) == (ch is None)
        m = sp.csr_matrix(m)
        m.sort_indices()
        m.eliminate_zeros()
        np.testing.assert_array_equal(ip.numpy(), m.indptr)
        np.testing.assert_array_equal(ix.numpy(), m.indices)
        np.testing.assert_array_equal(v.numpy(), m.data)   # same summation order: same bits
        assert ip.numel() == n + 1


def test_device_term_groups_dictionary_layout_deduplicates_complex128():
    """Summed in a fixed order, equal complex128 entries keep equal bits, so the
    dictionary of (column - row, value) pairs is as small as the host one."""
    from qutip_gb300.operator import dict_sliced_layout
    from qutip_gb300.superop import device_dict_layout, device_term_groups, sliced_padding
    from qutip_gb300.systems import merge_terms
    terms = _split_terms(5)
    dev = device_term_groups(terms, device="cpu")
    assert sliced_padding(dev) <= 1.15
    n = terms[0][0].shape[0]
    lay_d = device_dict_layout(dev, n, "c128")
    lay_h = dict_sliced_layout([m for m, _ in merge_terms(terms)], n, "c128")
    assert lay_d is not None and lay_h is not None
    assert lay_d[-1] == lay_h[-1]                                  # stored entries
    assert int(lay_d[5].numel()) == len(lay_h[5])                  # table entries
    np.testing.assert_array_equal(lay_d[6].numpy(), lay_h[6])      # table starts per group
