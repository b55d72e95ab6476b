"""A small straight-line SSA language for the step's pointwise functions, with
reverse-mode code generation.

A pointwise function (one face's Roe flux, one cell's PLM edge states, ...) is
written once as a Python function over ``Sym`` values.  Running it on symbolic
inputs records a list of SSA statements.  Branches are written as ``select``
on recorded conditions, so every statement executes and a branch decision is a
plain boolean value, which the reverse code replays.

From one trace the emitters produce:

* ``emit_numpy``: a NumPy function (forward, or forward + reverse sweep) over
  arrays -- elementwise, so the operation order and rounding of each statement
  are those of the trace;
* ``emit_cuda``: ``__device__`` functions ``<name>_fwd`` and ``<name>_rev`` for
  one item, in the same statement order (built without FMA contraction they
  round exactly like the NumPy version).

The reverse sweep is the textbook adjoint of each statement, emitted in reverse
order after a forward recomputation, with adjoints kept only for statements that
both depend on an input and reach an output.
"""
from __future__ import annotations

import math
import re


class Trace:
    def __init__(self, name):
        self.name = name
        self.nodes = []          # (op, args, meta)
        self.inputs = []         # node ids of differentiable inputs
        self.params = []         # node ids of non-differentiable parameters
        self.outputs = []        # node ids (or Python floats) of outputs
        self.consts = {}

    # -- node creation -----------------------------------------------------
    def _add(self, op, args, meta=None, kind="f"):
        self.nodes.append((op, tuple(args), meta, kind))
        return len(self.nodes) - 1

    def const(self, x):
        x = float(x)
        key = x.hex()
        if key not in self.consts:
            self.consts[key] = self._add("const", (), x)
        return Sym(self, self.consts[key])

    def input(self, n):
        out = []
        for _ in range(n):
            i = self._add("input", (), len(self.inputs))
            self.inputs.append(i)
            out.append(Sym(self, i))
        return out

    def param(self, n):
        out = []
        for _ in range(n):
            i = self._add("param", (), len(self.params))
            self.params.append(i)
            out.append(Sym(self, i))
        return out

    def set_outputs(self, outs):
        self.outputs = [self._lift(o).id for o in outs]

    def _lift(self, x):
        if isinstance(x, Sym):
            return x
        return self.const(x)


class Sym:
    __slots__ = ("t", "id")

    def __init__(self, t, i):
        self.t = t
        self.id = i

    def _bin(self, op, o, rev=False):
        o = self.t._lift(o)
        a, b = (o, self) if rev else (self, o)
        return Sym(self.t, self.t._add(op, (a.id, b.id)))

    def __add__(self, o): return self._bin("add", o)
    def __radd__(self, o): return self._bin("add", o, True)
    def __sub__(self, o): return self._bin("sub", o)
    def __rsub__(self, o): return self._bin("sub", o, True)
    def __mul__(self, o): return self._bin("mul", o)
    def __rmul__(self, o): return self._bin("mul", o, True)
    def __truediv__(self, o): return self._bin("div", o)
    def __rtruediv__(self, o): return self._bin("div", o, True)
    def __neg__(self): return Sym(self.t, self.t._add("neg", (self.id,)))

    def _cmp(self, op, o):
        o = self.t._lift(o)
        return Cond(self.t, self.t._add(op, (self.id, o.id), kind="b"))

    def __gt__(self, o): return self._cmp("gt", o)
    def __ge__(self, o): return self._cmp("ge", o)
    def __lt__(self, o): return self._cmp("lt", o)
    def __le__(self, o): return self._cmp("le", o)
    def eq(self, o): return self._cmp("eq", o)


class Cond:
    __slots__ = ("t", "id")

    def __init__(self, t, i):
        self.t = t
        self.id = i

    def __and__(self, o): return Cond(self.t, self.t._add("and", (self.id, o.id), kind="b"))
    def __or__(self, o): return Cond(self.t, self.t._add("or", (self.id, o.id), kind="b"))
    def __invert__(self): return Cond(self.t, self.t._add("not", (self.id,), kind="b"))


def sqrt(x): return Sym(x.t, x.t._add("sqrt", (x.id,)))
def fabs(x): return Sym(x.t, x.t._add("abs", (x.id,)))


def select(c, a, b):
    """c ? a : b (both sides are evaluated; the reverse sweep follows c)."""
    t = c.t
    a = t._lift(a)
    b = t._lift(b)
    return Sym(t, t._add("sel", (c.id, a.id, b.id)))


def dmax(a, b):
    """numpy.maximum on non-NaN data: a > b ? a : b."""
    t = a.t if isinstance(a, Sym) else b.t
    a, b = t._lift(a), t._lift(b)
    return select(a > b, a, b)


def dmin(a, b):
    t = a.t if isinstance(a, Sym) else b.t
    a, b = t._lift(a), t._lift(b)
    return select(a < b, a, b)


def trace(name, fn, n_in, n_par, **kw):
    """Record fn(inputs, params, **kw) -> outputs into a Trace."""
    t = Trace(name)
    ins = t.input(n_in)
    pars = t.param(n_par)
    outs = fn(ins, pars, **kw)
    t.set_outputs(list(outs))
    return t


# ----------------------------------------------------------------------------
# analysis
# ----------------------------------------------------------------------------
def _active(t):
    n = len(t.nodes)
    dep = [False] * n        # depends on a differentiable input
    for i, (op, args, meta, kind) in enumerate(t.nodes):
        if op == "input":
            dep[i] = True
        elif kind == "f" and op not in ("const", "param"):
            if op == "sel":
                dep[i] = dep[args[1]] or dep[args[2]]
            else:
                dep[i] = any(dep[a] for a in args)
    reach = [False] * n      # reaches an output
    for o in t.outputs:
        reach[o] = True
    for i in range(n - 1, -1, -1):
        if not reach[i]:
            continue
        op, args, meta, kind = t.nodes[i]
        if kind != "f":
            continue
        if op == "sel":
            reach[args[1]] = True
            reach[args[2]] = True
        else:
            for a in args:
                if t.nodes[a][3] == "f":
                    reach[a] = True
    return [dep[i] and reach[i] for i in range(n)]


def _live_forward(t, need):
    """Nodes whose forward value is needed (for outputs and for the reverse sweep)."""
    n = len(t.nodes)
    live = [False] * n
    for i in need:
        live[i] = True
    for i in range(n - 1, -1, -1):
        if live[i]:
            for a in t.nodes[i][1]:
                live[a] = True
    return live


def _reverse_needs(t, act):
    """Forward values the reverse sweep reads."""
    need = set()
    for i, (op, args, meta, kind) in enumerate(t.nodes):
        if not act[i] or kind != "f":
            continue
        if op == "mul":
            need.update(args)
        elif op == "div":
            need.update(args)
            need.add(i)
        elif op == "sqrt":
            need.add(i)
        elif op == "abs":
            need.add(args[0])
        elif op == "sel":
            need.add(args[0])
    return need


# ----------------------------------------------------------------------------
# emitters
# ----------------------------------------------------------------------------
_PY_BIN = {"add": "+", "sub": "-", "mul": "*", "div": "/"}
_C_RN = {"add": "__dadd_rn", "sub": "__dsub_rn", "mul": "__dmul_rn", "div": "DSL_FDIV"}
_CMP = {"gt": ">", "ge": ">=", "lt": "<", "le": "<=", "eq": "=="}
# CUDA comparisons on the IEEE bit pattern (``dsl_*`` in the emitted preamble): an FP64
# compare issues on the FP64 pipe at the DFMA rate, the pattern test on the integer pipe;
# both agree for every non-NaN operand, zeros of either sign included
_C_CMP = {op: f"dsl_{op}" for op in _CMP}
_C_PREAMBLE = (
    "#ifndef MHD_DSL_NZ\n#define MHD_DSL_NZ\n"
    "#include \"mhd_math.cuh\"\n"

    "__device__ __forceinline__ bool nz(double x) { return (__double_as_longlong(x) << 1) != 0; }\n"
    "__device__ __forceinline__ long long dsl_key(double x) {\n"
    "  const long long b = __double_as_longlong(x);\n"
    "  return b < 0 ? (-0x7fffffffffffffffLL - 1) - b : b;\n"
    "}\n"
    "__device__ __forceinline__ bool dsl_gt(double a, double b) { return dsl_key(a) > dsl_key(b); }\n"
    "__device__ __forceinline__ bool dsl_ge(double a, double b) { return dsl_key(a) >= dsl_key(b); }\n"
    "__device__ __forceinline__ bool dsl_lt(double a, double b) { return dsl_key(a) < dsl_key(b); }\n"
    "__device__ __forceinline__ bool dsl_le(double a, double b) { return dsl_key(a) <= dsl_key(b); }\n"
    "__device__ __forceinline__ bool dsl_eq(double a, double b) { return dsl_key(a) == dsl_key(b); }\n"
    "__device__ __forceinline__ bool dsl_pos(double x) { return __double_as_longlong(x) > 0; }\n"
    "__device__ __forceinline__ bool dsl_nonneg(double x) { return dsl_key(x) >= 0; }\n"
    # b / v for the reverse statements, which need not round like NumPy: Newton-Raphson
    # refinement of the reciprocal (r <- r + r(1 - v r), error squared per step) from the
    # hardware estimate (PTX rcp.approx.ftz.f64), then one residual correction of the
    # quotient q <- q + r(b - v q) (Markstein's final step), which multiplies the
    # quotient's error by the reciprocal's.  One refinement step (DSL_RDIV_STEPS) already
    # keeps the result within two ulps (tested); a second one measured 1.5% slower in the
    # backward pass.  Divisors whose exponent lies outside [2^-1000, 2^1000] (zero,
    # subnormal, huge, inf, NaN) take the correctly rounded division, so those keep its
    # IEEE results.
    "#ifndef DSL_RDIV_STEPS\n#define DSL_RDIV_STEPS 1\n#endif\n"
    "__device__ __forceinline__ double dsl_div(double b, double v) {\n"
    "  const unsigned int ex = ((unsigned int)__double2hiint(v) >> 20) & 0x7ffu;\n"
    "  if (ex - 23u > 2000u) return b / v;\n"
    "  double r;\n"
    "  asm(\"rcp.approx.ftz.f64 %0, %1;\" : \"=d\"(r) : \"d\"(v));\n"
    "  double e = fma(-v, r, 1.0);\n"
    "  r = fma(r, e, r);\n"
    "#if DSL_RDIV_STEPS > 1\n"
    "  e = fma(-v, r, 1.0);\n"
    "  r = fma(r, e, r);\n"
    "#endif\n"
    "  const double q = b * r;\n"
    "  return fma(r, fma(-v, q, b), q);\n"
    "}\n"
    "#endif")


def _fwd_lines(t, live, lang):
    L = []
    for i, (op, args, meta, kind) in enumerate(t.nodes):
        if not live[i]:
            continue
        v = f"v{i}"
        a = [f"v{x}" for x in args]
        if op == "const":
            lit = repr(meta) if lang == "py" else _c_lit(meta)
            L.append((v, lit, kind))
        elif op == "input":
            L.append((v, f"x[{meta}]", kind))
        elif op == "param":
            L.append((v, f"p[{meta}]", kind))
        elif op in _PY_BIN:
            if lang == "py":
                L.append((v, f"{a[0]} {_PY_BIN[op]} {a[1]}", kind))
            elif op == "div" and t.nodes[args[1]][0] == "const" and t.nodes[args[1]][2] == 6.0:
                # correctly rounded x / 6 without an IEEE division (mhdk::div6)
                L.append((v, f"mhdk::div6({a[0]})", kind))
            elif op == "div" and t.nodes[args[1]][0] == "const" and _pow2(t.nodes[args[1]][2]):
                # x / 2^k and x * 2^-k are the same real number, rounded once
                L.append((v, f"__dmul_rn({a[0]}, {_c_lit(1.0 / t.nodes[args[1]][2])})", kind))
            else:
                # round-to-nearest intrinsics are never contracted into an FMA, so
                # the forward values round exactly like NumPy's even in a unit
                # compiled with contraction on (the reverse statements use it)
                L.append((v, f"{_C_RN[op]}({a[0]}, {a[1]})", kind))
        elif op == "neg":
            L.append((v, f"-{a[0]}", kind))
        elif op == "sqrt":
            L.append((v, f"np.sqrt({a[0]})" if lang == "py" else f"DSL_FSQRT({a[0]})", kind))
        elif op == "abs":
            L.append((v, f"np.abs({a[0]})" if lang == "py" else f"fabs({a[0]})", kind))
        elif op in _CMP:
            L.append((v, f"{a[0]} {_CMP[op]} {a[1]}" if lang == "py" else f"{_C_CMP[op]}({a[0]}, {a[1]})", kind))
        elif op == "and":
            L.append((v, f"{a[0]} & {a[1]}" if lang == "py" else f"{a[0]} && {a[1]}", kind))
        elif op == "or":
            L.append((v, f"{a[0]} | {a[1]}" if lang == "py" else f"{a[0]} || {a[1]}", kind))
        elif op == "not":
            L.append((v, f"~{a[0]}" if lang == "py" else f"!{a[0]}", kind))
        elif op == "sel":
            L.append((v, f"np.where({a[0]}, {a[1]}, {a[2]})" if lang == "py" else f"{a[0]} ? {a[1]} : {a[2]}", kind))
        else:
            raise ValueError(op)
    return L


def _pow2(x):
    """x is +-2^k with 2^-k a normal double."""
    m, e = math.frexp(abs(x))
    return x != 0.0 and m == 0.5 and -1021 <= 1 - e <= 1022


def _c_lit(x):
    if math.isinf(x) or math.isnan(x):
        raise ValueError("non-finite constant")
    r = repr(float(x))
    if "e" not in r and "." not in r and "inf" not in r:
        r += ".0"
    return r


def _rev_lines_c(t, act, first_of=None):
    """CUDA adjoint statements in reverse order.  b{i} is the adjoint of node i.

    Each adjoint is declared by its first contribution (no zero start, so no
    extra addition).  Only a contribution that multiplies the incoming adjoint
    by a forward value is guarded by ``nz(b)``: a branch not taken may hold a
    non-finite value (e.g. w/bt with bt == 0) and 0 * inf must not reach the
    result.  Sums, differences and selects pass the adjoint through unguarded.
    A quotient's two contributions share one division, and the divisions of the
    quotient and square-root rules go through ``dsl_div`` (a refined reciprocal,
    within two ulps of the correctly rounded quotient); a constant divisor becomes
    a multiply by its reciprocal.  These statements may contract into FMAs: the
    adjoint is not required to round like the NumPy reverse sweep.
    """
    L = []
    declared = set() if first_of is None else first_of

    def acc(j, expr, guard=None, neg=False):
        if not act[j]:
            return
        if j not in declared:
            declared.add(j)
            e = f"-({expr})" if neg else expr
            L.append(f"double b{j} = {guard} ? {e} : 0.0" if guard else f"double b{j} = {e}")
        else:
            op = "-=" if neg else "+="
            L.append(f"if ({guard}) b{j} {op} {expr}" if guard else f"b{j} {op} {expr}")

    for k, o in enumerate(t.outputs):
        if act[o]:
            acc(o, f"ybar[{k}]")
    for i in range(len(t.nodes) - 1, -1, -1):
        op, args, meta, kind = t.nodes[i]
        if not act[i] or kind != "f" or op == "input":
            continue
        b = f"b{i}"
        if op == "add":
            acc(args[0], b)
            acc(args[1], b)
        elif op == "sub":
            acc(args[0], b)
            acc(args[1], b, neg=True)
        elif op == "neg":
            acc(args[0], b, neg=True)
        elif op == "mul":
            if act[args[0]] or act[args[1]]:
                L.append(f"const bool g{i} = nz({b})")
            acc(args[0], f"{b} * v{args[1]}", guard=f"g{i}")
            acc(args[1], f"{b} * v{args[0]}", guard=f"g{i}")
        elif op == "div":
            # the quotient may be non-finite on a branch not taken: guard its use
            L.append(f"const bool g{i} = nz({b})")
            if t.nodes[args[1]][0] == "const" and t.nodes[args[1]][2] != 0.0:
                # a constant divisor: multiply by its reciprocal (within an ulp)
                L.append(f"const double q{i} = {b} * {_c_lit(1.0 / t.nodes[args[1]][2])}")
            else:
                L.append(f"const double q{i} = g{i} ? dsl_div({b}, v{args[1]}) : 0.0")
            acc(args[0], f"q{i}")
            acc(args[1], f"q{i} * v{i}", guard=f"g{i}", neg=True)
        elif op == "sqrt":
            acc(args[0], f"dsl_div(0.5 * {b}, v{i})", guard=f"(nz({b}) && dsl_pos(v{i}))")
        elif op == "abs":
            acc(args[0], f"(dsl_nonneg(v{args[0]}) ? {b} : -{b})")
        elif op == "sel":
            acc(args[1], f"(v{args[0]} ? {b} : 0.0)")
            acc(args[2], f"(v{args[0]} ? 0.0 : {b})")
        else:
            raise ValueError(op)
    return L


def _rev_lines(t, act, lang):
    """Adjoint statements in reverse order.  b{i} is the adjoint of node i."""
    L = []
    where = (lambda c, x: f"np.where({c}, {x}, 0.0)") if lang == "py" else (lambda c, x: f"({c} ? {x} : 0.0)")
    for i in range(len(t.nodes) - 1, -1, -1):
        op, args, meta, kind = t.nodes[i]
        if not act[i] or kind != "f" or op == "input":
            continue
        b = f"b{i}"

        # contributions are skipped when the incoming adjoint is exactly zero, so a
        # non-finite value on a branch not taken (e.g. w/bt with bt == 0) never
        # turns into 0 * inf
        def acc(j, expr):
            if act[j]:
                if lang == "py":
                    L.append(f"b{j} = b{j} + np.where({b} != 0.0, {expr}, 0.0)")
                else:
                    L.append(f"if (nz({b})) b{j} = b{j} + ({expr})")

        if op == "add":
            acc(args[0], b)
            acc(args[1], b)
        elif op == "sub":
            acc(args[0], b)
            acc(args[1], f"-{b}")
        elif op == "mul":
            acc(args[0], f"{b} * v{args[1]}")
            acc(args[1], f"{b} * v{args[0]}")
        elif op == "div":
            acc(args[0], f"{b} / v{args[1]}")
            acc(args[1], f"-({b} * v{i}) / v{args[1]}")
        elif op == "neg":
            acc(args[0], f"-{b}")
        elif op == "sqrt":
            acc(args[0], where(f"v{i} > 0.0", f"({b} * 0.5) / v{i}"))
        elif op == "abs":
            acc(args[0], f"np.where(v{args[0]} >= 0.0, {b}, -{b})" if lang == "py"
                else f"(dsl_nonneg(v{args[0]}) ? {b} : -{b})")
        elif op == "sel":
            acc(args[1], where(f"v{args[0]}", b))
            nc = f"~v{args[0]}" if lang == "py" else f"!v{args[0]}"
            acc(args[2], where(nc, b))
        else:
            raise ValueError(op)
    return L


def emit_numpy(t, reverse=False):
    """Python source of ``fwd(x, p) -> outs`` (and ``rev(x, p, ybar) -> xbar``) over NumPy arrays."""
    act = _active(t)
    need_out = set(t.outputs)
    src = [f"def {t.name}_fwd(x, p):", "    with np.errstate(all='ignore'):"]
    live = _live_forward(t, need_out)
    for v, e, kind in _fwd_lines(t, live, "py"):
        src.append(f"        {v} = {e}")
    src.append("    return [" + ", ".join(f"v{o}" for o in t.outputs) + "]")
    if reverse:
        need = need_out | _reverse_needs(t, act)
        live = _live_forward(t, need)
        src.append("")
        src.append(f"def {t.name}_rev(x, p, ybar):")
        src.append("    with np.errstate(all='ignore'):")
        for v, e, kind in _fwd_lines(t, live, "py"):
            src.append(f"        {v} = {e}")
        for i in range(len(t.nodes)):
            if act[i] and t.nodes[i][3] == "f":
                src.append(f"        b{i} = 0.0")
        for k, o in enumerate(t.outputs):
            if act[o]:
                src.append(f"        b{o} = b{o} + ybar[{k}]")
        for line in _rev_lines(t, act, "py"):
            src.append("        " + line)
        xb = []
        for i in t.inputs:
            xb.append(f"b{i}" if act[i] else "0.0")
        src.append("    return [" + ", ".join(xb) + "]")
    return "\n".join(src) + "\n"


def _reverse_needs_c(t, act):
    """Forward values the CUDA reverse statements (``_rev_lines_c``) read."""
    need = set()
    for i, (op, args, meta, kind) in enumerate(t.nodes):
        if not act[i] or kind != "f":
            continue
        if op == "mul":
            if act[args[0]]:
                need.add(args[1])
            if act[args[1]]:
                need.add(args[0])
        elif op == "div":
            need.add(args[1])
            if act[args[1]]:
                need.add(i)
        elif op == "sqrt":
            need.add(i)
        elif op == "abs":
            need.add(args[0])
        elif op == "sel":
            need.add(args[0])
    return need


def tape_layout(t):
    """(float nodes, bool nodes) the reverse sweep reads that are computed, not inputs,
    parameters or constants: what a forward sweep stores on the tape."""
    need = _reverse_needs_c(t, _active(t))
    fl = sorted(i for i in need if t.nodes[i][3] == "f" and t.nodes[i][0] not in ("input", "param", "const"))
    bl = sorted(i for i in need if t.nodes[i][3] == "b")
    return fl, bl


def tape_words(t):
    fl, bl = tape_layout(t)
    return len(fl) + (len(bl) + 31) // 32


def branch_layout(t):
    """Every branch decision of a forward sweep, in node order: each live condition
    node, and the sign of each live |x| (the kink of the absolute value).  A forward
    sweep that records these bits and one that replays them (``emit_cuda``'s
    ``_fwdb<1>`` / ``_fwdb<2>``) evaluate the same smooth piece of the function at
    nearby inputs -- the piece whose derivative the reverse sweep returns."""
    live = _live_forward(t, set(t.outputs))
    return [i for i, (op, args, meta, kind) in enumerate(t.nodes) if live[i] and (kind == "b" or op == "abs")]


def branch_words(t):
    return (len(branch_layout(t)) + 31) // 32


def emit_cuda(t, reverse=True):
    """CUDA source for one item of a traced function:

    * ``<name>_fwd(x, p, y)``: forward;
    * ``<name>_rev(x, p, ybar, xbar)``: forward recomputation, then the reverse sweep;
    * ``<name>_fwdt(x, p, y, tape, stride)``: forward that also stores the values
      the reverse sweep reads (``tape_layout``) at tape[k * stride] (booleans
      packed 32 to a word);
    * ``<name>_revt(x, p, ybar, xbar, tape, stride)``: the reverse sweep reading
      those values back instead of recomputing the forward.
    """
    act = _active(t)
    need_out = set(t.outputs)
    out = []
    live = _live_forward(t, need_out)
    out.append(_C_PREAMBLE)
    out.append(f"__device__ __forceinline__ void {t.name}_fwd(const double* __restrict__ x, "
               f"const double* __restrict__ p, double* __restrict__ y) {{")
    for v, e, kind in _fwd_lines(t, live, "c"):
        ty = "double" if kind == "f" else "bool"
        out.append(f"  const {ty} {v} = {e};")
    for k, o in enumerate(t.outputs):
        out.append(f"  y[{k}] = v{o};")
    out.append("}")
    out.append(_emit_branch_forward(t, live))
    if not reverse:
        return "\n".join(out) + "\n"
    need = need_out | _reverse_needs_c(t, act)
    live = _live_forward(t, need)
    out.append(f"__device__ __forceinline__ void {t.name}_rev(const double* __restrict__ x, "
               f"const double* __restrict__ p, const double* __restrict__ ybar, double* __restrict__ xbar) {{")
    for v, e, kind in _fwd_lines(t, live, "c"):
        ty = "double" if kind == "f" else "bool"
        out.append(f"  const {ty} {v} = {e};")
    declared = set()
    for line in _rev_lines_c(t, act, declared):
        out.append("  " + line + ";")
    for k, i in enumerate(t.inputs):
        out.append(f"  xbar[{k}] = {'b%d' % i if i in declared else '0.0'};")
    out.append("}")
    # taped pair
    fl, bl = tape_layout(t)
    fslot = {i: k for k, i in enumerate(fl)}
    bslot = {i: (len(fl) + k // 32, k % 32) for k, i in enumerate(bl)}
    nbw = (len(bl) + 31) // 32
    live_out = _live_forward(t, need_out | set(fl) | set(bl))
    out.append(f"__device__ __forceinline__ void {t.name}_fwdt(const double* __restrict__ x, "
               f"const double* __restrict__ p, double* __restrict__ y, double* __restrict__ tape, size_t stride) {{")
    for w in range(nbw):
        out.append(f"  unsigned int tw{w} = 0u;")
    for v, e, kind in _fwd_lines(t, live_out, "c"):
        ty = "double" if kind == "f" else "bool"
        out.append(f"  const {ty} {v} = {e};")
        i = int(v[1:])
        if i in fslot:
            out.append(f"  tape[{fslot[i]} * stride] = {v};")
        elif i in bslot:
            w, bit = bslot[i]
            out.append(f"  tw{w - len(fl)} |= (unsigned int){v} << {bit};")
    for w in range(nbw):
        out.append(f"  tape[{len(fl) + w} * stride] = __hiloint2double(0, (int)tw{w});")
    for k, o in enumerate(t.outputs):
        out.append(f"  y[{k}] = v{o};")
    out.append("}")
    out.append(f"__device__ __forceinline__ void {t.name}_revt(const double* __restrict__ x, "
               f"const double* __restrict__ p, const double* __restrict__ ybar, double* __restrict__ xbar, "
               f"const double* __restrict__ tape, size_t stride) {{")
    # each forward value is loaded right before the first reverse statement that
    # reads it, which keeps live ranges (and register pressure) short
    loaded, words_loaded = set(), set()

    def load(i):
        op, args, meta, kind = t.nodes[i]
        if op == "input":
            return [f"const double v{i} = x[{meta}]"]
        if op == "param":
            return [f"const double v{i} = p[{meta}]"]
        if op == "const":
            return [f"const double v{i} = {_c_lit(meta)}"]
        if i in fslot:
            return [f"const double v{i} = tape[{fslot[i]} * stride]"]
        w, bit = bslot[i]
        pre = []
        if w not in words_loaded:
            words_loaded.add(w)
            pre.append(f"const unsigned int tw{w - len(fl)} = (unsigned int)__double2loint(tape[{w} * stride])")
        return pre + [f"const bool v{i} = (tw{w - len(fl)} >> {bit}) & 1u"]

    declared = set()
    for line in _rev_lines_c(t, act, declared):
        for m in re.findall(r"\bv(\d+)\b", line):
            i = int(m)
            if i not in loaded:
                loaded.add(i)
                for ld in load(i):
                    out.append("  " + ld + ";")
        out.append("  " + line + ";")
    for k, i in enumerate(t.inputs):
        out.append(f"  xbar[{k}] = {'b%d' % i if i in declared else '0.0'};")
    out.append("}")
    return "\n".join(out) + "\n"


def _emit_branch_forward(t, live):
    """``<name>_fwdb<MODE>(x, p, y, bt, stride)``: the forward sweep with its branch
    decisions (``branch_layout``) on a bit tape of 32-bit words at bt[k * stride].
    MODE 1 records them; MODE 2 replays them -- each condition takes its recorded
    value and each |x| its recorded sign -- so that the sweep stays on the piece of
    the function it was on when they were recorded."""
    bl = branch_layout(t)
    bslot = {i: (k // 32, k % 32) for k, i in enumerate(bl)}
    nw = (len(bl) + 31) // 32
    out = [f"template <int MODE>",
           f"__device__ __forceinline__ void {t.name}_fwdb(const double* __restrict__ x, "
           f"const double* __restrict__ p, double* __restrict__ y, unsigned int* __restrict__ bt, size_t stride) {{"]
    for w in range(nw):
        out.append(f"  unsigned int bw{w} = MODE == 2 ? bt[{w} * stride] : 0u;")
    if nw == 0:
        out.append("  (void)bt; (void)stride;")
    for v, e, kind in _fwd_lines(t, live, "c"):
        i = int(v[1:])
        ty = "double" if kind == "f" else "bool"
        if i not in bslot:
            out.append(f"  const {ty} {v} = {e};")
            continue
        w, bit = bslot[i]
        op, args, meta, _ = t.nodes[i]
        if kind == "b":
            out.append(f"  const bool {v} = MODE == 2 ? (((bw{w} >> {bit}) & 1u) != 0u) : ({e});")
            out.append(f"  if (MODE == 1) bw{w} |= (unsigned int){v} << {bit};")
        else:  # |x|: the sign of x is the decision
            a = f"v{args[0]}"
            out.append(f"  const bool s{i} = MODE == 2 ? (((bw{w} >> {bit}) & 1u) != 0u) : dsl_nonneg({a});")
            out.append(f"  if (MODE == 1) bw{w} |= (unsigned int)s{i} << {bit};")
            out.append(f"  const double {v} = s{i} ? {a} : -{a};")
    if nw:
        out.append("  if (MODE == 1) {")
        for w in range(nw):
            out.append(f"    bt[{w} * stride] = bw{w};")
        out.append("  }")
    for k, o in enumerate(t.outputs):
        out.append(f"  y[{k}] = v{o};")
    out.append("}")
    return "\n".join(out)


def emit_torch(t):
    """Python source of ``fwd(x, p) -> outs`` over torch tensors (forward only, for
    torch's own automatic differentiation)."""
    live = _live_forward(t, set(t.outputs))
    src = [f"def {t.name}_fwd(x, p):"]
    for i, (op, args, meta, kind) in enumerate(t.nodes):
        if not live[i]:
            continue
        a = [f"v{x}" for x in args]
        if op == "const":
            e = repr(meta)
        elif op == "input":
            e = f"x[{meta}]"
        elif op == "param":
            e = f"p[{meta}]"
        elif op == "div":
            e = f"_div({a[0]}, {a[1]})"
        elif op in _PY_BIN:
            e = f"_t({a[0]}) {_PY_BIN[op]} _t({a[1]})"
        elif op == "neg":
            e = f"-{a[0]}"
        elif op == "sqrt":
            e = f"_sqrt({a[0]})"
        elif op == "abs":
            e = f"_abs({a[0]})"
        elif op in _CMP:
            e = f"_t({a[0]}) {_CMP[op]} {a[1]}"
        elif op == "and":
            e = f"{a[0]} & {a[1]}"
        elif op == "or":
            e = f"{a[0]} | {a[1]}"
        elif op == "not":
            e = f"~{a[0]}"
        elif op == "sel":
            e = f"_where({a[0]}, {a[1]}, {a[2]})"
        else:
            raise ValueError(op)
        src.append(f"    v{i} = {e}")
    src.append("    return [" + ", ".join(f"v{o}" for o in t.outputs) + "]")
    return "\n".join(src) + "\n"


_TORCH_SQRT = None


def _torch_sqrt():
    """Correctly rounded float64 square root for torch tensors with its derivative
    rules (reverse and forward mode).  torch's CPU sqrt is not correctly rounded;
    the value comes from NumPy on the host, or from torch on a CUDA device, where
    sqrt is IEEE round-to-nearest."""
    global _TORCH_SQRT
    if _TORCH_SQRT is None:
        import numpy as np
        import torch

        class Sqrt(torch.autograd.Function):
            @staticmethod
            def forward(x):
                if x.is_cuda:
                    return torch.sqrt(x)
                return torch.from_numpy(np.sqrt(x.detach().numpy()))

            @staticmethod
            def setup_context(ctx, inputs, output):
                ctx.save_for_backward(output)
                ctx.save_for_forward(output)

            @staticmethod
            def backward(ctx, g):
                (y,) = ctx.saved_tensors
                return g * (0.5 / y)

            @staticmethod
            def jvp(ctx, t):
                (y,) = ctx.saved_tensors
                return t * (0.5 / y)

        _TORCH_SQRT = Sqrt.apply
    return _TORCH_SQRT


def compile_torch(t, device=None):
    """Executable torch forward function of a trace on ``device``.

    Constants become tensors on that device: torch computes a tensor divided by a
    host scalar through the scalar's reciprocal, which rounds differently.
    Quotients and square roots use the masked ("double where") form, so torch's
    reverse mode never forms 0 * inf on a branch not taken: the divisor or
    radicand is replaced by 1 where it is zero (not positive, for the root) and
    the value by 0 there -- the same convention as the hand-written reverse
    sweeps, and the same values wherever a result is finite.  |x| is
    differentiated as +1 at 0, like the hand-written sweeps.
    """
    import torch

    dev = torch.device(device) if device is not None else torch.device("cpu")

    def _t(x):
        return x if isinstance(x, torch.Tensor) else torch.tensor(x, dtype=torch.float64, device=dev)

    def _where(c, a, b):
        return torch.where(c, _t(a), _t(b))

    sq = _torch_sqrt()

    def _div(a, b):
        a, b = _t(a), _t(b)
        z = b == 0.0
        return torch.where(z, 0.0, a / torch.where(z, 1.0, b))

    def _sqrt(x):
        x = _t(x)
        pos = x > 0.0
        return torch.where(pos, sq(torch.where(pos, x, 1.0)), x * 0.0)

    def _abs(x):
        x = _t(x)
        return torch.where(x >= 0.0, x, -x)

    ns = {"_sqrt": _sqrt, "_abs": _abs, "_t": _t, "_where": _where, "_div": _div}
    exec(compile(emit_torch(t), f"<dsl-torch:{t.name}>", "exec"), ns)
    return ns[f"{t.name}_fwd"]


def compile_numpy(t, reverse=False):
    """Executable (fwd[, rev]) NumPy functions of a trace."""
    import numpy as np
    ns = {"np": np}
    exec(compile(emit_numpy(t, reverse), f"<dsl:{t.name}>", "exec"), ns)
    if reverse:
        return ns[f"{t.name}_fwd"], ns[f"{t.name}_rev"]
    return ns[f"{t.name}_fwd"]
