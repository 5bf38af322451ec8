"""Custom propensity expressions as stack bytecode.

The reference turns a reaction's ``propensity_function`` string into C++
(``Model.expr.getexpr_cpp``, spatialpy/solvers/build_expression.py:308-324)
and compiles it into the generated model file as
``double f(const int *x, double t, const double vol, const double *data_fn,
int sd)`` (spatialpy/solvers/solver.py:344-373), with species as ``x[i]``,
parameters as constants, ``vol`` the particle volume, ``t`` the time and
``sd`` the particle type.  Here the same Python expression is compiled into
a small postfix program that the event kernels (and the CPU oracle)
evaluate in double precision, rounding the result to float like every other
propensity:

=========  ====================================================
opcode     meaning
=========  ====================================================
END        stop; the value is the top of the stack
CONST k    push constant k (index into the constants table)
X s        push the count of species s
VOL, T     push vol (m/rho), the time
TYPE       push the particle type
DATA i     push data function i at the particle
ADD..POW   binary arithmetic; POWI n: integer power by products
NEG        unary minus
EXP..CEIL  math functions (exp, log, sqrt, sin, cos, tan, fabs,
           log10, floor, ceil)
LT..NE     comparisons, 1.0 / 0.0
AND, OR    non-zero tests, 1.0 / 0.0; NOT likewise
=========  ====================================================

Programs hold at most ``MAX_STACK`` values; the engine rechecks the depth
of every program before using it.
"""
from __future__ import annotations

import ast
import math

import numpy as np

END, CONST, X, VOL, T, TYPE, DATA = 0, 1, 2, 3, 4, 5, 6
ADD, SUB, MUL, DIV, POW, NEG, POWI = 10, 11, 12, 13, 14, 15, 16
EXP, LOG, SQRT, SIN, COS, TAN, FABS, LOG10, FLOOR, CEIL = 20, 21, 22, 23, 24, 25, 26, 27, 28, 29
LT, LE, GT, GE, EQ, NE, AND, OR, NOT = 30, 31, 32, 33, 34, 35, 36, 37, 38
MAX_STACK = 16

_FUNCS = {"exp": EXP, "log": LOG, "sqrt": SQRT, "sin": SIN, "cos": COS, "tan": TAN,
          "fabs": FABS, "abs": FABS, "log10": LOG10, "floor": FLOOR, "ceil": CEIL}
_BIN = {ast.Add: ADD, ast.Sub: SUB, ast.Mult: MUL, ast.Div: DIV, ast.Pow: POW}
_CMP = {ast.Lt: LT, ast.LtE: LE, ast.Gt: GT, ast.GtE: GE, ast.Eq: EQ, ast.NotEq: NE}


class PropensityError(ValueError):
    """An expression this compiler does not accept."""


def compile_expression(expr: str, species: list, constants: dict, consts: list,
                       data_names: list = ()) -> list:
    """Compile one propensity expression.

    species: species names (their index is the X operand); constants: name
    -> value (parameters, and any fixed names); consts: the shared constants
    table, extended in place; data_names: data functions (DATA operand).
    Returns the program as a list of int words.
    """
    didx = {d: i for i, d in enumerate(data_names)}
    tree = ast.parse(expr.strip(), mode="eval")
    code: list = []
    sidx = {s: i for i, s in enumerate(species)}

    def const(v):
        v = float(v)
        for i, c in enumerate(consts):
            if c == v and math.copysign(1.0, c) == math.copysign(1.0, v):
                code.extend([CONST, i])
                return
        consts.append(v)
        code.extend([CONST, len(consts) - 1])

    def emit(node):
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)) \
                and not isinstance(node.value, bool):
            const(node.value)
        elif isinstance(node, ast.Name):
            n = node.id
            if n in sidx:
                code.extend([X, sidx[n]])
            elif n == "vol":
                code.append(VOL)
            elif n == "t":
                code.append(T)
            elif n == "sd":
                code.append(TYPE)
            elif n in didx:
                code.extend([DATA, didx[n]])
            elif n in constants:
                const(constants[n])
            elif n in ("pi", "e"):
                const(getattr(math, n))
            else:
                raise PropensityError(f"unknown name {n!r} in propensity {expr!r}")
        elif isinstance(node, ast.BinOp) and type(node.op) in _BIN:
            if isinstance(node.op, ast.Pow) and _int_const(node.right) is not None:
                emit(node.left)
                code.extend([POWI, _int_const(node.right)])
            else:
                emit(node.left)
                emit(node.right)
                code.append(_BIN[type(node.op)])
        elif isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
            emit(node.operand)
            code.append(NEG)
        elif isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.UAdd):
            emit(node.operand)
        elif isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.Not):
            emit(node.operand)
            code.append(NOT)
        elif isinstance(node, ast.Call) and isinstance(node.func, ast.Name) \
                and node.func.id in _FUNCS and len(node.args) == 1 and not node.keywords:
            emit(node.args[0])
            code.append(_FUNCS[node.func.id])
        elif isinstance(node, ast.Call) and isinstance(node.func, ast.Name) \
                and node.func.id == "pow" and len(node.args) == 2:
            if _int_const(node.args[1]) is not None:
                emit(node.args[0])
                code.extend([POWI, _int_const(node.args[1])])
            else:
                emit(node.args[0])
                emit(node.args[1])
                code.append(POW)
        elif isinstance(node, ast.Compare) and len(node.ops) == 1 and type(node.ops[0]) in _CMP:
            emit(node.left)
            emit(node.comparators[0])
            code.append(_CMP[type(node.ops[0])])
        elif isinstance(node, ast.BoolOp):
            emit(node.values[0])
            for v in node.values[1:]:
                emit(v)
                code.append(AND if isinstance(node.op, ast.And) else OR)
        else:
            raise PropensityError(f"unsupported construct {ast.dump(node)[:60]} in {expr!r}")

    emit(tree.body)
    code.append(END)
    depth = stack_depth(code)
    if depth > MAX_STACK:
        raise PropensityError(f"propensity {expr!r} needs a stack of {depth} (> {MAX_STACK})")
    return code


def _int_const(node):
    if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)) \
            and not isinstance(node.value, bool):
        v = node.value
        if float(v).is_integer() and abs(v) <= 64:
            return int(v)
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
        v = _int_const(node.operand)
        return None if v is None else -v
    return None


def stack_depth(code) -> int:
    """Largest stack of a program; raises on underflow or a missing END."""
    d = best = 0
    pc = 0
    while pc < len(code):
        op = code[pc]
        if op == END:
            if d != 1:
                raise PropensityError("program leaves %d values" % d)
            return best
        if op in (CONST, X, DATA):
            d += 1
            pc += 2
        elif op in (VOL, T, TYPE):
            d += 1
            pc += 1
        elif op == POWI:
            if d < 1:
                raise PropensityError("stack underflow")
            pc += 2
        elif op in (NEG, NOT) or EXP <= op <= CEIL:
            if d < 1:
                raise PropensityError("stack underflow")
            pc += 1
        elif ADD <= op <= POW or LT <= op <= OR:
            if d < 2:
                raise PropensityError("stack underflow")
            d -= 1
            pc += 1
        else:
            raise PropensityError(f"bad opcode {op}")
        best = max(best, d)
    raise PropensityError("program without END")


def evaluate(code, consts, x, vol: float, t: float = 0.0, typ: int = 1, data=()) -> float:
    """Reference evaluation in Python double precision (test use); data:
    this particle's data function values."""
    st = []
    pc = 0
    f = {EXP: math.exp, LOG: math.log, SQRT: math.sqrt, SIN: math.sin, COS: math.cos,
         TAN: math.tan, FABS: math.fabs, LOG10: math.log10, FLOOR: math.floor, CEIL: math.ceil}
    while True:
        op = code[pc]
        if op == END:
            return st[-1]
        if op == CONST:
            st.append(consts[code[pc + 1]]); pc += 2
        elif op == X:
            st.append(float(x[code[pc + 1]])); pc += 2
        elif op == VOL:
            st.append(vol); pc += 1
        elif op == T:
            st.append(t); pc += 1
        elif op == TYPE:
            st.append(float(typ)); pc += 1
        elif op == DATA:
            st.append(float(data[code[pc + 1]])); pc += 2
        elif op == POWI:
            st.append(_powi(st.pop(), code[pc + 1])); pc += 2
        elif op == NEG:
            st.append(-st.pop()); pc += 1
        elif op == NOT:
            st.append(1.0 if st.pop() == 0.0 else 0.0); pc += 1
        elif op in f:
            st.append(f[op](st.pop())); pc += 1
        else:
            b, a = st.pop(), st.pop()
            st.append({ADD: lambda: a + b, SUB: lambda: a - b, MUL: lambda: a * b,
                       DIV: lambda: a / b, POW: lambda: math.pow(a, b),
                       LT: lambda: float(a < b), LE: lambda: float(a <= b),
                       GT: lambda: float(a > b), GE: lambda: float(a >= b),
                       EQ: lambda: float(a == b), NE: lambda: float(a != b),
                       AND: lambda: float(a != 0.0 and b != 0.0),
                       OR: lambda: float(a != 0.0 or b != 0.0)}[op]())
            pc += 1


def _powi(a: float, n: int) -> float:
    """a**n by repeated products in a fixed order (the kernels' order)."""
    m = -n if n < 0 else n
    r = 1.0
    for _ in range(m):
        r = r * a
    return 1.0 / r if n < 0 else r


def mass_action_ode(k: float, reactants: list, consts: list) -> list:
    """The deterministic rate of a mass-action reaction (reaction.py:283-300):
    ``k * A * B`` or ``k * A * A``, left to right; reactants: (species
    index, stoichiometry) pairs."""
    code = []
    v = float(k)
    if v in consts:
        code.extend([CONST, consts.index(v)])
    else:
        consts.append(v)
        code.extend([CONST, len(consts) - 1])
    for s, n in reactants:
        for _ in range(n):
            code.extend([X, s, MUL])
    code.append(END)
    return code


def pack(programs: list):
    """Concatenate per-reaction programs: (code int32, offsets int64 [R+1])."""
    off = [0]
    words = []
    for p in programs:
        words.extend(p if p is not None else [])
        off.append(len(words))
    return np.array(words, np.int32), np.array(off, np.int64)
