"""Shared pytest configuration: the ``gpu`` marker and fixture loading helpers."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def csr_from(g, prefix):
    import scipy.sparse as sp
    shape = tuple(int(v) for v in g[f"{prefix}_shape"]) if f"{prefix}_shape" in g else None
    n = len(g[f"{prefix}_indptr"]) - 1
    return sp.csr_matrix((g[f"{prefix}_data"], g[f"{prefix}_indices"], g[f"{prefix}_indptr"]),
                         shape=shape or (n, n))


def pcg_state(row):
    """Rebuild a numpy PCG64 generator from the stored 128-bit state/increment."""
    row = [int(v) for v in row]
    g = np.random.Generator(np.random.PCG64())
    g.bit_generator.state = {"bit_generator": "PCG64",
                             "state": {"state": (row[0] << 64) | row[1], "inc": (row[2] << 64) | row[3]},
                             "has_uint32": 0, "uinteger": 0}
    return g


def jump_records_match(got_t, got_w, g, tr):
    """Same jump count and channels, each time inside the reference's own bisection
    window (recorded per jump in the golden fixture)."""
    o0, o1 = int(g["col_off"][tr]), int(g["col_off"][tr + 1])
    want_t, want_w, win = g["col_times"][o0:o1], g["col_which"][o0:o1], g["col_window"][o0:o1]
    if len(got_t) != len(want_t) or [int(w) for w in got_w] != [int(w) for w in want_w]:
        return False
    return bool(np.all(np.abs(np.asarray(got_t) - want_t) <= win))


def jump_times_close(got_t, g, tr, tol=1e-6):
    o0, o1 = int(g["col_off"][tr]), int(g["col_off"][tr + 1])
    return len(got_t) == o1 - o0 and np.allclose(got_t, g["col_times"][o0:o1], rtol=tol, atol=tol)
