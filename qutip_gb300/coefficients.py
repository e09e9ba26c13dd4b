"""Time-dependent coefficients compiled to a bytecode the device evaluates.

The reference evaluates each term's coefficient ``c_k(t)`` on the host once per
right-hand-side call (``_BaseElement.matmul_data_t``,
qutip/core/cy/_element.pyx:166-182).  Coefficients given as strings are compiled
by Cython at run time (qutip/core/coefficient.py:399-450) and the combinators
``Conj``/``Sum``/``Mul``/``Constant`` live in qutip/core/cy/coefficient.pyx:688-950.

Here a coefficient becomes a small stack program over complex doubles.  The
device evaluates it at every stage time inside the kernels, so a time-dependent
right-hand side needs no host round trip.  The host parses the expression with
:mod:`ast` once; ``args`` are folded in as constants.

Program layout (shared with ``csrc/coeff_vm.cuh``): an ``int32`` code stream
where ``OP_CONST`` is followed by an index into the ``complex128`` constant pool.
"""
from __future__ import annotations

import ast
import cmath
import math
from typing import Mapping

import numpy as np

__all__ = ["Coefficient", "coefficient", "interpolation", "OPCODES", "MAX_STACK",
           "pack_programs"]

OPCODES = {
    "END": 0, "CONST": 1, "T": 2, "ADD": 3, "SUB": 4, "MUL": 5, "DIV": 6, "NEG": 7,
    "COS": 8, "SIN": 9, "EXP": 10, "LOG": 11, "SQRT": 12, "CONJ": 13, "REAL": 14,
    "IMAG": 15, "ABS": 16, "POW": 17, "COSH": 18, "SINH": 19, "TANH": 20, "TAN": 21,
    "ARCTAN": 22, "INTERP": 23,
}
MAX_STACK = 16
_FUNCS = {"cos": "COS", "sin": "SIN", "exp": "EXP", "log": "LOG", "sqrt": "SQRT",
          "conj": "CONJ", "conjugate": "CONJ", "real": "REAL", "imag": "IMAG",
          "abs": "ABS", "cosh": "COSH", "sinh": "SINH", "tanh": "TANH", "tan": "TAN",
          "arctan": "ARCTAN"}
_NAMES = {"pi": math.pi, "e": math.e, "j": 1j}
_BINOPS = {ast.Add: "ADD", ast.Sub: "SUB", ast.Mult: "MUL", ast.Div: "DIV", ast.Pow: "POW"}


class Coefficient:
    """A device-evaluable scalar function ``c(t)``.

    ``code``/``consts`` are the program; ``expr`` is a human-readable form.
    """

    def __init__(self, code, consts, expr: str):
        self.code = [int(c) for c in code]
        self.consts = [complex(c) for c in consts]
        self.expr = expr
        if self.code[-1] != OPCODES["END"]:
            self.code.append(OPCODES["END"])
        depth = _max_depth(self.code)
        if depth > MAX_STACK:
            raise ValueError(f"coefficient {expr!r} needs stack depth {depth} > {MAX_STACK}")

    # -- algebra (mirrors Conj/Sum/Mul coefficients) ------------------------
    def _body(self):
        return self.code[:-1]

    def _combine(self, other: "Coefficient", op: str, sym: str) -> "Coefficient":
        shift = len(self.consts)
        body2 = _shift_consts(other._body(), shift)
        return Coefficient(self._body() + body2 + [OPCODES[op]],
                           self.consts + other.consts, f"({self.expr}){sym}({other.expr})")

    def conj(self) -> "Coefficient":
        """``conj(c)``; a program that is real for every real t is its own conjugate, so
        it comes back unchanged (the reference's ConjCoefficient of a real function --
        the spost part of every Liouvillian with a real time dependence -- then shares
        the original's coefficient group)."""
        if self.is_real():
            return self
        return Coefficient(self._body() + [OPCODES["CONJ"]], self.consts, f"conj({self.expr})")

    def is_real(self) -> bool:
        """Whether the program returns a real number for every real t: a static pass over
        the stack that tracks, per slot, whether the value is provably real.  Real
        constants and t are real; +, -, *, /, negation, cos, sin, exp, cosh, sinh, tanh,
        tan, arctan and conj keep realness; real, imag and abs always give a real value;
        log, sqrt, pow (a negative real argument gives a complex result) and
        interpolation are treated as possibly complex."""
        keep = {OPCODES[k] for k in ("NEG", "COS", "SIN", "EXP", "COSH", "SINH", "TANH", "TAN",
                                     "ARCTAN", "CONJ")}
        make = {OPCODES[k] for k in ("REAL", "IMAG", "ABS")}
        binary = {OPCODES[k] for k in ("ADD", "SUB", "MUL", "DIV")}
        stack: list[bool] = []
        i = 0
        code = self.code
        while i < len(code):
            op = code[i]
            if op == OPCODES["END"]:
                break
            if op == OPCODES["CONST"]:
                stack.append(self.consts[code[i + 1]].imag == 0)
                i += 2
                continue
            if op == OPCODES["INTERP"]:
                stack.append(False)
                i += 2
                continue
            if op == OPCODES["T"]:
                stack.append(True)
            elif op in keep:
                pass
            elif op in make:
                stack[-1] = True
            elif op in binary:
                b = stack.pop()
                stack[-1] = stack[-1] and b
            else:                       # LOG, SQRT, POW and anything unknown
                if op == OPCODES["POW"]:
                    stack.pop()
                stack[-1] = False
            i += 1
        return len(stack) == 1 and stack[0]

    def __add__(self, other):
        return self._combine(_as_coeff(other), "ADD", "+")

    def __mul__(self, other):
        return self._combine(_as_coeff(other), "MUL", "*")

    __radd__ = __add__
    __rmul__ = __mul__

    def key(self):
        return (tuple(self.code), tuple(self.consts))

    def __call__(self, t: float) -> complex:
        """Run the program on the host (used to check the device interpreter)."""
        return _run(self.code, self.consts, float(t))

    def __repr__(self):
        return f"Coefficient({self.expr!r})"


def _as_coeff(x) -> Coefficient:
    return x if isinstance(x, Coefficient) else coefficient(x)


def _shift_consts(code, shift):
    out, i = [], 0
    while i < len(code):
        out.append(code[i])
        if code[i] in (OPCODES["CONST"], OPCODES["INTERP"]):
            out.append(code[i + 1] + shift)
            i += 1
        i += 1
    return out


def _max_depth(code):
    d = best = 0
    i = 0
    unary = {OPCODES[k] for k in ("NEG", "COS", "SIN", "EXP", "LOG", "SQRT", "CONJ", "REAL",
                                  "IMAG", "ABS", "COSH", "SINH", "TANH", "TAN", "ARCTAN")}
    while i < len(code):
        op = code[i]
        if op == OPCODES["END"]:
            break
        if op in (OPCODES["CONST"], OPCODES["INTERP"]):
            d += 1
            i += 1
        elif op == OPCODES["T"]:
            d += 1
        elif op in unary:
            pass
        else:
            d -= 1
        best = max(best, d)
        i += 1
    return best


class _Compiler(ast.NodeVisitor):
    def __init__(self, args: Mapping):
        self.args = dict(args or {})
        self.code: list[int] = []
        self.consts: list[complex] = []

    def const(self, v):
        v = complex(v)
        if v in self.consts:
            idx = self.consts.index(v)
        else:
            idx = len(self.consts)
            self.consts.append(v)
        self.code += [OPCODES["CONST"], idx]

    def visit_Expression(self, node):
        self.visit(node.body)

    def visit_Constant(self, node):
        if not isinstance(node.value, (int, float, complex)) or isinstance(node.value, bool):
            raise ValueError(f"unsupported literal {node.value!r}")
        self.const(node.value)

    def visit_Name(self, node):
        if node.id == "t":
            self.code.append(OPCODES["T"])
        elif node.id in self.args:
            v = self.args[node.id]
            if not np.isscalar(v):
                raise ValueError(f"argument {node.id!r} must be a scalar number")
            self.const(v)
        elif node.id in _NAMES:
            self.const(_NAMES[node.id])
        else:
            raise ValueError(f"unknown name {node.id!r} in coefficient")

    def visit_Attribute(self, node):
        # np.pi / numpy.pi
        if isinstance(node.value, ast.Name) and node.value.id in ("np", "numpy", "math", "cmath"):
            if node.attr in _NAMES:
                return self.const(_NAMES[node.attr])
        raise ValueError(f"unsupported attribute {ast.unparse(node)!r}")

    def visit_UnaryOp(self, node):
        self.visit(node.operand)
        if isinstance(node.op, ast.USub):
            self.code.append(OPCODES["NEG"])
        elif not isinstance(node.op, ast.UAdd):
            raise ValueError("unsupported unary operator")

    def visit_BinOp(self, node):
        op = _BINOPS.get(type(node.op))
        if op is None:
            raise ValueError(f"unsupported operator {type(node.op).__name__}")
        self.visit(node.left)
        self.visit(node.right)
        self.code.append(OPCODES[op])

    def visit_Call(self, node):
        f = node.func
        name = f.attr if isinstance(f, ast.Attribute) else getattr(f, "id", None)
        if name not in _FUNCS or len(node.args) != 1 or node.keywords:
            raise ValueError(f"unsupported function call {ast.unparse(node)!r}")
        self.visit(node.args[0])
        self.code.append(OPCODES[_FUNCS[name]])

    def generic_visit(self, node):
        raise ValueError(f"unsupported syntax {type(node).__name__}")


def coefficient(base, args: Mapping | None = None) -> Coefficient:
    """Build a :class:`Coefficient` from a number, a string expression or a Coefficient.

    Strings follow the reference's string-coefficient syntax
    (qutip/core/coefficient.py:63-130): a Python expression in ``t`` and the
    names in ``args``, using ``cos, sin, exp, log, sqrt, conj, real, imag, abs,
    cosh, sinh, tanh, tan, arctan`` (optionally prefixed ``np.``), ``pi`` and
    ``1j``.
    """
    if isinstance(base, Coefficient):
        return base
    if isinstance(base, (int, float, complex, np.number)):
        return Coefficient([OPCODES["CONST"], 0, OPCODES["END"]], [complex(base)], repr(base))
    if isinstance(base, str):
        comp = _Compiler(args)
        comp.visit(ast.parse(base.strip(), mode="eval"))
        a = ", ".join(f"{k}={v!r}" for k, v in sorted((args or {}).items()))
        return Coefficient(comp.code + [OPCODES["END"]], comp.consts, f"{base} [{a}]")
    raise TypeError(f"cannot evaluate a coefficient of type {type(base).__name__} on the device")


def _cpow(a: complex, b: complex) -> complex:
    """a ** b as the device interpreter evaluates it (``eval_coef``): real pow for a real
    base and exponent when the base is positive or the exponent an integer (0 ** -k is
    inf), 0 for any other zero base, exp(b log a) otherwise."""
    if a.imag == 0.0 and b.imag == 0.0 and (a.real > 0.0 or b.real == math.floor(b.real)):
        if a.real == 0.0 and b.real < 0.0:
            return complex(math.inf)
        return complex(a.real ** b.real)
    if a == 0:
        return 0j
    return cmath.exp(b * cmath.log(a))


def _run(code, consts, t):
    st: list[complex] = []
    i = 0
    O = OPCODES
    un = {O["COS"]: cmath.cos, O["SIN"]: cmath.sin, O["EXP"]: cmath.exp, O["LOG"]: cmath.log,
          O["SQRT"]: cmath.sqrt, O["CONJ"]: lambda z: z.conjugate(), O["REAL"]: lambda z: z.real,
          O["IMAG"]: lambda z: z.imag, O["ABS"]: abs, O["COSH"]: cmath.cosh,
          O["SINH"]: cmath.sinh, O["TANH"]: cmath.tanh, O["TAN"]: cmath.tan,
          O["ARCTAN"]: cmath.atan, O["NEG"]: lambda z: -z}
    while True:
        op = code[i]
        if op == O["END"]:
            break
        if op == O["CONST"]:
            i += 1
            st.append(consts[code[i]])
        elif op == O["INTERP"]:
            i += 1
            st.append(_interp_eval(consts, code[i], t))
        elif op == O["T"]:
            st.append(complex(t))
        elif op in un:
            st.append(complex(un[op](st.pop())))
        else:
            b, a = st.pop(), st.pop()
            if op == O["ADD"]:
                st.append(a + b)
            elif op == O["SUB"]:
                st.append(a - b)
            elif op == O["MUL"]:
                st.append(a * b)
            elif op == O["DIV"]:
                st.append(a / b if b != 0 else complex("nan"))
            elif op == O["POW"]:
                st.append(_cpow(a, b))
            else:
                raise ValueError(f"unknown opcode {op}")
        i += 1
    return st[-1]


def interpolation(tlist, poly, dt=0.0) -> Coefficient:
    """A piecewise polynomial ``poly[order+1][n]`` on breakpoints ``tlist`` (the form
    of the reference's ``InterCoefficient``, qutip/core/cy/coefficient.pyx:412-566):
    ``poly[order][0]`` below the first breakpoint, ``poly[order][n-1]`` from the last,
    Horner in ``t - tlist[idx]`` inside; ``dt`` non-zero marks uniform breakpoints."""
    tl = np.asarray(tlist, dtype=np.float64).reshape(-1)
    pl = np.asarray(poly, dtype=np.complex128)
    if pl.ndim != 2 or pl.shape[1] != tl.shape[0] or tl.shape[0] == 0:
        raise ValueError("poly must have shape (order + 1, len(tlist))")
    n, order = tl.shape[0], pl.shape[0] - 1
    consts = [complex(n, order), complex(float(dt), 0.0)] + [complex(x) for x in tl] + \
        [complex(z) for z in pl.reshape(-1)]
    return Coefficient([OPCODES["INTERP"], 0, OPCODES["END"]], consts,
                       f"interp(n={n}, order={order})")


def _interp_eval(consts, k, t):
    n, order = int(consts[k].real), int(consts[k].imag)
    dt = consts[k + 1].real
    tl = [consts[k + 2 + i].real for i in range(n)]
    base = k + 2 + n

    def p(i, j):
        return consts[base + i * n + j]
    if t <= tl[0]:
        return p(order, 0)
    if t >= tl[-1]:
        return p(order, n - 1)
    if dt != 0.0:
        idx = int((t - tl[0]) / dt)
    else:
        lo, hi, count = 0, n, 0
        while lo + 1 != hi and count < 64:
            mid = (lo + hi) // 2
            if t < tl[mid]:
                hi = mid
            else:
                lo = mid
            count += 1
        idx = lo
    idx = min(max(idx, 0), n - 1)
    if order == 0:
        return p(0, idx)
    f = t - tl[idx]
    out = 0j
    for i in range(order + 1):
        out = out * f + p(i, idx)
    return out


def pack_programs(coeffs):
    """Concatenate per-group programs for the device.

    Returns ``(code int32[], starts int32[G+1], consts float64[2*K])``; a ``None``
    coefficient becomes the constant 1.
    """
    code: list[int] = []
    starts = [0]
    consts: list[complex] = []
    for c in coeffs:
        c = coefficient(1.0) if c is None else c
        code += _shift_consts(c._body(), len(consts)) + [OPCODES["END"]]
        consts += c.consts
        starts.append(len(code))
    cz = np.zeros(2 * max(len(consts), 1), dtype=np.float64)
    for i, z in enumerate(consts):
        cz[2 * i], cz[2 * i + 1] = z.real, z.imag
    return (np.asarray(code, dtype=np.int32), np.asarray(starts, dtype=np.int32), cz)
