"""Build ``libqutip_gb300.so`` (sm_103a) from ``csrc/`` with nvcc, in-tree.

The library is a plain shared object with a C ABI (``include/qutip_gb300.h``);
the host layer loads it with ctypes.  Translation units compile in parallel and
are rebuilt only when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
GEN = BUILD / "gen"
LIB = PKG / "libqutip_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def generate_tableau() -> Path:
    """Write the Vern7 tableau header from ``vern7_tableau.py`` (single source of truth)."""
    sys.path.insert(0, str(ROOT))
    from qutip_gb300 import vern7_tableau as T
    GEN.mkdir(parents=True, exist_ok=True)
    a = [[0.0] * 16 for _ in range(16)]
    for i, row in enumerate(T.A):
        a[i][:len(row)] = row
    h = lambda x: float(x).hex()  # noqa: E731
    arr1 = lambda v: "{" + ", ".join(h(x) for x in v) + "}"  # noqa: E731
    arr2 = lambda m: "{" + ", ".join(arr1(r) for r in m) + "}"  # noqa: E731
    # float pairs hi + lo with hi = fl32(x), lo = fl32(x - hi) (about 48 significant bits)
    import numpy as np
    f32 = lambda x: float(np.float32(x))  # noqa: E731
    hi = lambda v: [f32(x) for x in v]  # noqa: E731
    lo = lambda v: [f32(x - f32(x)) for x in v]  # noqa: E731
    fa1 = lambda v: "{" + ", ".join(float(x).hex() + "f" if x else "0.0f" for x in v) + "}"  # noqa: E731
    fa2 = lambda m: "{" + ", ".join(fa1(r) for r in m) + "}"  # noqa: E731
    src = f"""// Generated from qutip_gb300/vern7_tableau.py by qutip_gb300/build.py.  Do not edit.
#pragma once
namespace qg {{
constexpr int RK_STEP = {T.RK_STEP};
constexpr int RK_EXTRA_STEP = {T.RK_EXTRA_STEP};
constexpr int DENSE_ORDER = {T.DENSEOUT_ORDER};
constexpr int RK_ORDER = {T.ORDER};
static __constant__ double VERN7_A[16][16] = {arr2(a)};
static __constant__ double VERN7_B[10] = {arr1(T.B)};
static __constant__ double VERN7_C[16] = {arr1(T.C)};
static __constant__ double VERN7_E[10] = {arr1(T.E)};
static __constant__ double VERN7_BI[16][7] = {arr2(T.BI)};
static __constant__ float VERN7_AH[16][16] = {fa2([hi(r) for r in a])};
static __constant__ float VERN7_AL[16][16] = {fa2([lo(r) for r in a])};
static __constant__ float VERN7_BH[10] = {fa1(hi(T.B))};
static __constant__ float VERN7_BL[10] = {fa1(lo(T.B))};
static __constant__ float VERN7_EF[10] = {fa1(hi(T.E))};
static __constant__ float VERN7_EL[10] = {fa1(lo(T.E))};
static const double VERN7_A_HOST[16][16] = {arr2(a)};
static const double VERN7_B_HOST[10] = {arr1(T.B)};
static const double VERN7_C_HOST[16] = {arr1(T.C)};
static const double VERN7_E_HOST[10] = {arr1(T.E)};
static const double VERN7_BI_HOST[16][7] = {arr2(T.BI)};
}}  // namespace qg
"""
    out = GEN / "vern7_tableau.cuh"
    if not out.exists() or out.read_text() != src:
        out.write_text(src)
    return out


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [ROOT / "include" / "qutip_gb300.h", PKG / "vern7_tableau.py",
                                   Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    generate_tableau()
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    objdir = BUILD / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    inc = ["-I", str(ROOT / "include"), "-I", str(GEN), "-I", str(CSRC)]

    def one(src: Path):
        obj = objdir / (src.stem + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *inc, "-c", str(src), "-o", str(obj)]
        p = subprocess.run(cmd, capture_output=True, text=True)
        return src, obj, p

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(one, _sources()))
    failed = [r for r in results if r[2].returncode != 0]
    for src, _, p in results:
        if verbose or p.returncode != 0:
            sys.stderr.write(f"== {src.name}\n{p.stdout}{p.stderr}")
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(r[0].name for r in failed))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(r[1]) for r in results], "-lcudart"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("link failed:\n" + p.stdout + p.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
