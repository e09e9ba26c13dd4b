"""Build recipe for ``oracle/_ref``: the reference QuTiP compiled from its own sources.

TEST INFRASTRUCTURE ONLY.  The compiled reference is the checker and the timed
CPU baseline; nothing in ``qutip_gb300`` imports or executes it.

The reference ships a meson-python build (``meson.build``, ``qutip/meson.build``)
that cannot run without network access.  This recipe reproduces what that build
does, in two stages, so that the expensive Cython step runs where Cython is
installed and the C++ step runs on whichever machine (x86_64 or aarch64) will
import the result:

``prepare``   (needs the reference checkout and Cython)
    * copy the ``qutip`` package to ``oracle/_ref/qutip`` (outputs stay under
      ``oracle/_ref``, which is git-ignored);
    * write ``qutip/core/data/src/intdtype.h`` with 32-bit ``idxint`` -- the
      file ``qutip/meson.build:1-22`` generates with the default
      ``idxint_64=false`` (``meson.options:4-9``);
    * cythonize every module listed in ``qutip/meson.build:28-40`` (C++
      language, ``meson.build:7-12``) into ``.cpp`` next to its ``.pyx``;
    * write a ``qutip-<ver>.dist-info/METADATA`` because ``qutip/__init__.py:9``
      asks ``importlib.metadata`` for the version.

``compile``   (needs g++, Python headers and numpy headers)
    * compile every generated ``.cpp`` into an extension module with the flags
      of ``meson.build:14-21`` (``-O3 -funroll-loops -std=c++17``); the
      ``matmul`` module also links the three hand-written kernels
      (``qutip/meson.build:55-64``).

Usage::

    python oracle/build_ref.py prepare     # here
    python oracle/build_ref.py compile     # here and on any other host
    python oracle/build_ref.py all
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

REF_ROOT = Path(os.environ.get("QUTIP_REFERENCE_ROOT", "/root/reference"))
OUT = Path(__file__).resolve().parent / "_ref"
PKG = OUT / "qutip"

# qutip/meson.build:28-40 (the ``cy_modules`` table) plus the matmul module.
CY_MODULES = {
    ".": ["_distributions"],
    "core": ["_brtools", "_brtensor"],
    "core/cy": ["_element", "coefficient", "lindblad_matrix_form", "math", "qobjevo"],
    "core/data": ["add", "adjoint", "base", "block_operations", "convert", "csr",
                  "data_iterator", "dense", "dia", "dispatch", "expect", "inner",
                  "kron", "_local_matmul", "mean", "mul", "norm", "ode", "permute",
                  "pow", "project", "properties", "ptrace", "reshape", "tidyup",
                  "trace", "matmul"],
    "piqs": ["_piqs"],
    "solver/cy": ["dysolve", "nm_mcsolve"],
    "solver/integrator": ["explicit_rk", "_rhs"],
    "solver/sode": ["_sode", "ssystem"],
}
MATMUL_EXTRA = ["core/data/src/matmul_csr_vector.cpp",
                "core/data/src/matmul_csr_dense.cpp",
                "core/data/src/matmul_diag_vector.cpp"]
CXXFLAGS = ["-O3", "-funroll-loops", "-std=c++17", "-fPIC", "-shared", "-w",
            "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION"]


def _version() -> str:
    v = (REF_ROOT / "VERSION").read_text().strip() if (REF_ROOT / "VERSION").exists() else "5.4.0"
    return v.replace("dev", ".dev0") if "dev" in v and ".dev" not in v else v


def prepare() -> None:
    from Cython.Build import cythonize  # only needed for this stage

    if not (REF_ROOT / "qutip").is_dir():
        raise SystemExit(f"reference checkout not found at {REF_ROOT}")
    if PKG.exists():
        shutil.rmtree(PKG)
    OUT.mkdir(parents=True, exist_ok=True)
    shutil.copytree(REF_ROOT / "qutip", PKG,
                    ignore=shutil.ignore_patterns("__pycache__", "*.so", ".pytest_cache"))
    (PKG / "core/data/src/intdtype.h").write_text(
        "typedef int32_t idxint;\nstatic const int _idxint_size = 32;\n")
    pyx = [str(PKG / d / f"{m}.pyx") for d, mods in CY_MODULES.items() for m in mods]
    cwd = os.getcwd()
    os.chdir(OUT)
    try:
        cythonize([os.path.relpath(p, OUT) for p in pyx], language_level=3,
                  compiler_directives={"language_level": 3}, nthreads=os.cpu_count() or 4,
                  include_path=[str(OUT), str(PKG / "core/data")], force=True, quiet=True,
                  language="c++")
    finally:
        os.chdir(cwd)
    ver = _version()
    dist = OUT / f"qutip-{ver}.dist-info"
    dist.mkdir(exist_ok=True)
    (dist / "METADATA").write_text(f"Metadata-Version: 2.1\nName: qutip\nVersion: {ver}\n")
    (dist / "top_level.txt").write_text("qutip\n")


def _compile_one(d: str, m: str) -> tuple[str, int, str]:
    import numpy

    src = PKG / d / f"{m}.cpp"
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    dst = PKG / d / f"{m}{ext}"
    if dst.exists() and dst.stat().st_mtime > src.stat().st_mtime:
        return (f"{d}/{m}", 0, "up to date")
    srcs = [str(src)]
    if m == "matmul":
        srcs += [str(PKG / s) for s in MATMUL_EXTRA]
    cmd = (["g++"] + CXXFLAGS + [f"-I{sysconfig.get_paths()['include']}",
                                 f"-I{numpy.get_include()}", f"-I{PKG / 'core/data'}",
                                 f"-I{PKG / 'core/data/src'}"] + srcs + ["-o", str(dst)])
    p = subprocess.run(cmd, capture_output=True, text=True)
    return (f"{d}/{m}", p.returncode, p.stderr[-2000:])


def compile_all() -> None:
    if not PKG.is_dir():
        raise SystemExit("oracle/_ref/qutip missing: run `prepare` where Cython is installed")
    jobs = [(d, m) for d, mods in CY_MODULES.items() for m in mods]
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        res = list(ex.map(lambda a: _compile_one(*a), jobs))
    bad = [r for r in res if r[1] != 0]
    for name, rc, err in bad:
        print(f"FAILED {name} rc={rc}\n{err}", file=sys.stderr)
    if bad:
        raise SystemExit(1)


def available() -> bool:
    """True when a compiled reference for this interpreter exists under ``oracle/_ref``."""
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    return (PKG / "core/data" / f"matmul{ext}").exists()


if __name__ == "__main__":
    step = sys.argv[1] if len(sys.argv) > 1 else "all"
    if step in ("prepare", "all"):
        prepare()
    if step in ("compile", "all"):
        compile_all()
