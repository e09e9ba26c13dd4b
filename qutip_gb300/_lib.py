"""ctypes binding of ``libqutip_gb300.so`` (the C ABI in ``include/qutip_gb300.h``).

The library must be present: there is no CPU fallback.  Loading it needs no GPU;
any compute call on a machine without a CUDA device fails with the CUDA error the
library reports.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libqutip_gb300.so"

QG_OK, QG_ERR_ARG, QG_ERR_CUDA, QG_ERR_UNSUPPORTED = 0, -1, -2, -3
QG_C128, QG_C64 = 0, 1
QG_MAX_GROUPS, QG_MAX_EOPS, QG_MAX_COPS = 8, 32, 64


QG_LAYOUT_GROUP_MAJOR, QG_LAYOUT_ROW_MAJOR, QG_LAYOUT_SLICED, QG_LAYOUT_SLICED_DICT = 0, 1, 2, 3
QG_LAYOUT_SLICED_DICT_RI = 4
QG_DICT_MAX = 4096
QG_DENSE_MAX_D = 128
QG_TILE_ROWS = 512
QG_GROUP_AUTO, QG_GROUP_WARP, QG_GROUP_CTA, QG_GROUP_CLUSTER, QG_GROUP_CTA128 = 0, 1, 2, 3, 4


class CsrGroups(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("n_cols", C.c_int64), ("n_groups", C.c_int32),
                ("dtype", C.c_int32), ("layout", C.c_int32), ("lanes", C.c_int32),
                ("n_tiles", C.c_int32), ("tile_nnz", C.c_int32), ("row_ptr", C.c_void_p),
                ("col", C.c_void_p), ("val", C.c_void_p), ("tile_row", C.c_void_p),
                ("coef_code", C.c_void_p), ("coef_start", C.c_void_p),
                ("coef_consts", C.c_void_p), ("dict_off", C.c_void_p),
                ("dict_start", C.c_void_p)]


class Lindblad(C.Structure):
    _fields_ = [("d", C.c_int64), ("dtype", C.c_int32), ("n_groups", C.c_int32),
                ("n_diag_cops", C.c_int32), ("n_cops", C.c_int32),
                ("a_diag_const", C.c_int32), ("n_const_diag", C.c_int32),
                ("hermitian", C.c_int32), ("reserved", C.c_int32),
                ("a_width", C.c_int32 * QG_MAX_GROUPS), ("c_width", C.c_int32 * QG_MAX_COPS),
                ("d_const", C.c_void_p), ("a_diag", C.c_void_p), ("a_col", C.c_void_p), ("a_val", C.c_void_p),
                ("c_diag", C.c_void_p), ("c_col", C.c_void_p), ("c_val", C.c_void_p),
                ("a_coef_code", C.c_void_p), ("a_coef_start", C.c_void_p),
                ("a_coef_consts", C.c_void_p), ("c_coef_code", C.c_void_p),
                ("c_coef_start", C.c_void_p), ("c_coef_consts", C.c_void_p)]


class Sde(C.Structure):
    _fields_ = [("n", C.c_int64), ("open", C.c_int32), ("n_sc", C.c_int32), ("d", C.c_int32),
                ("reserved", C.c_int32), ("l_rp", C.c_void_p), ("l_col", C.c_void_p),
                ("l_val", C.c_void_p), ("c_rp", C.c_void_p), ("c_col", C.c_void_p),
                ("c_val", C.c_void_p), ("m_rp", C.c_void_p), ("m_col", C.c_void_p),
                ("m_val", C.c_void_p), ("work", C.c_void_p)]


class DenseLindblad(C.Structure):
    _fields_ = [("d", C.c_int32), ("n_groups", C.c_int32), ("n_cops", C.c_int32),
                ("reserved", C.c_int32), ("a", C.c_void_p), ("c", C.c_void_p),
                ("a_coef_code", C.c_void_p), ("a_coef_start", C.c_void_p),
                ("a_coef_consts", C.c_void_p), ("c_coef_code", C.c_void_p),
                ("c_coef_start", C.c_void_p), ("c_coef_consts", C.c_void_p)]


class Dia(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("n_cols", C.c_int64), ("n_diags", C.c_int32),
                ("dtype", C.c_int32), ("offsets", C.c_void_p), ("data", C.c_void_p)]


class RkBuffers(C.Structure):
    _fields_ = [("n", C.c_int64), ("state_dtype", C.c_int32), ("stage_dtype", C.c_int32),
                ("y_prev", C.c_void_p), ("y_front", C.c_void_p), ("y_prev_s", C.c_void_p),
                ("y_front_s", C.c_void_p), ("k", C.c_void_p),
                ("ytmp", C.c_void_p), ("scratch", C.c_void_p), ("counter", C.c_void_p),
                ("result", C.c_void_p)]


class StateView(C.Structure):
    _fields_ = [("n", C.c_int64), ("base_dtype", C.c_int32), ("k_dtype", C.c_int32),
                ("base", C.c_void_p), ("k", C.c_void_p), ("n_k", C.c_int32), ("pad_", C.c_int32),
                ("f", C.c_double * 16)]


_P = C.POINTER
_SIGS = {
    "qg_version": (C.c_int, []),
    "qg_last_error": (C.c_char_p, []),
    "qg_scratch_doubles": (C.c_int64, []),
    "qg_vern7_tableau": (C.c_int, [C.c_void_p] * 5),
    "qg_device_fault": (C.c_int, []),
    "qg_spmv_csr": (C.c_int, [_P(CsrGroups), C.c_double, C.c_void_p, C.c_void_p, C.c_double,
                              C.c_double, C.c_double, C.c_double, C.c_void_p]),
    "qg_spmm_csr": (C.c_int, [_P(CsrGroups), C.c_double, C.c_void_p, C.c_void_p, C.c_int64,
                              C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double,
                              C.c_void_p]),
    "qg_spmv_dia": (C.c_int, [_P(Dia), C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                              C.c_double, C.c_double, C.c_void_p]),
    "qg_vern7_stage": (C.c_int, [_P(CsrGroups), _P(RkBuffers), C.c_int, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_void_p]),
    "qg_lindblad_apply": (C.c_int, [_P(Lindblad), C.c_double, C.c_void_p, C.c_void_p,
                                    C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_void_p]),
    "qg_lindblad_stage": (C.c_int, [_P(Lindblad), _P(RkBuffers), C.c_int, C.c_double,
                                    C.c_double, C.c_double, C.c_double, C.c_void_p]),
    "qg_dense_lindblad_apply": (C.c_int, [_P(DenseLindblad), C.c_double, C.c_void_p, C.c_void_p,
                                          C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_void_p]),
    "qg_dense_lindblad_stage": (C.c_int, [_P(DenseLindblad), _P(RkBuffers), C.c_int, C.c_double,
                                          C.c_double, C.c_double, C.c_double, C.c_void_p]),
    "qg_sde_work_values": (C.c_int64, [C.c_int64, C.c_int32]),
    "qg_sde_platen": (C.c_int, [_P(Sde), C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                C.c_double, C.c_void_p]),
    "qg_sde_euler": (C.c_int, [_P(Sde), C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                               C.c_double, C.c_void_p]),
    "qg_rk_combine": (C.c_int, [_P(StateView), C.c_void_p, C.c_int, C.c_void_p]),
    "qg_norm2": (C.c_int, [C.c_void_p, C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                           C.c_void_p]),
    "qg_expect_dm": (C.c_int, [_P(CsrGroups), C.c_int64, _P(StateView), C.c_void_p, C.c_void_p]),
    "qg_expect_ket": (C.c_int, [_P(CsrGroups), _P(StateView), C.c_void_p, C.c_void_p]),
    "qg_abi_sizes": (C.c_int, [C.c_void_p, C.c_int]),
    "qg_batch_slot_bytes": (C.c_int64, [C.c_int64, C.c_int]),
    "qg_batch_max_slots": (C.c_int, [C.c_int64, C.c_int]),
    "qg_batch_group_slots": (C.c_int, [C.c_int64, C.c_int, C.c_int]),
    "qg_batch_launch_slots": (C.c_int, [C.c_void_p]),
    "qg_batch_smem_bytes": (C.c_int64, [C.c_void_p]),
    "qg_batch_vern7": (C.c_int, [C.c_void_p, C.c_void_p]),
    "qg_batch_vern7_noalloc": (C.c_int, [C.c_void_p, C.c_void_p]),
    "qg_batch_noalloc_staging_fault": (C.c_int, [C.c_void_p]),
}

_lib = None

# Entry points that launch exactly one kernel each; calls are counted so that a
# benchmark can report how many of this library's kernels ran in a timed region.
COMPUTE_ENTRY_POINTS = {
    "qg_spmv_csr", "qg_spmm_csr", "qg_spmv_dia", "qg_vern7_stage", "qg_rk_combine", "qg_norm2",
    "qg_expect_dm", "qg_expect_ket", "qg_batch_vern7", "qg_batch_vern7_noalloc",
    "qg_lindblad_apply", "qg_lindblad_stage", "qg_dense_lindblad_apply", "qg_dense_lindblad_stage",
    "qg_sde_platen", "qg_sde_euler",
}
LAUNCHES = [0]


class QgError(RuntimeError):
    pass


class _Counted:
    """The loaded library with kernel-launching entry points counted."""

    def __init__(self, lib):
        self._raw = lib

    def __getattr__(self, name):
        fn = getattr(self._raw, name)
        if name in COMPUTE_ENTRY_POINTS:
            def counted(*args, _fn=fn):
                LAUNCHES[0] += 1
                return _fn(*args)
            setattr(self, name, counted)
            return counted
        return fn


def load():
    """Load the shared library (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists() and os.environ.get("QUTIP_GB300_NO_BUILD") is None:
        from .build import build
        build()
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m qutip_gb300.build`")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = _Counted(lib)
    return _lib


def declared_symbols():
    return list(_SIGS)


def check(rc: int, what: str = ""):
    if rc == QG_OK:
        return
    msg = (load().qg_last_error() or b"").decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if rc == QG_ERR_ARG:
        raise ValueError(text)
    if rc == QG_ERR_UNSUPPORTED:
        raise TypeError(text)
    raise QgError(text)


def call(name: str, *args):
    check(getattr(load(), name)(*args), name)
