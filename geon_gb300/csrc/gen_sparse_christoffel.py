"""Generate sparse FP64 Christoffel symbols that are bit-identical to the dense
finite-difference fallback of the reference (metric/mod.rs:25-69 with
types.rs:34-47's inverse), for the metrics that use it (Alcubierre,
Morris-Thorne). Output: christoffel_sparse.cuh in this directory.

Method: run the dense algorithm symbolically. A value is an exact constant
(0, +-1), or a runtime expression. Only operations between runtime values, or
with constants other than 0 and +-1, are emitted, in the dense algorithm's
order. Rules (all exact in IEEE arithmetic for finite values):
  x*1 = x, x*(-1) = -x, 0*x = x*0 = 0 (up to the sign of zero),
  x + 0 = 0 + x = x, x - 0 = x, 0 - x = -x (up to the sign of zero),
  and a sum that starts at 0.0 (every sum of the reference does) never holds
  -0.0, so a zero term of either sign leaves it unchanged; the first nonzero
  term t gives 0.0 + t, emitted as plus_zero(t).
Results can differ from the dense code only in the sign of zero entries.
"""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))


class V:
    """Symbolic double: const in {0.0, 1.0, -1.0} or a C expression."""

    def __init__(self, const=None, expr=None):
        self.const, self.expr = const, expr

    def is_zero(self):
        return self.const == 0.0

    def c(self):
        if self.const is not None:
            return {0.0: "0.0", 1.0: "1.0", -1.0: "-1.0"}[self.const]
        return self.expr


ZERO, ONE, MONE = V(0.0), V(1.0), V(-1.0)


class Gen:
    def __init__(self):
        self.lines = []
        self.n = 0

    def tmp(self, expr):
        self.n += 1
        name = f"t{self.n}"
        self.lines.append(f"  const double {name} = {expr};")
        return V(expr=name)

    def neg(self, a):
        if a.const is not None:
            return V(-a.const) if a.const != 0.0 else ZERO
        return self.tmp(f"-{a.c()}")

    def mul(self, a, b):
        if a.is_zero() or b.is_zero():
            return ZERO
        if a.const == 1.0:
            return b
        if b.const == 1.0:
            return a
        if a.const == -1.0:
            return self.neg(b)
        if b.const == -1.0:
            return self.neg(a)
        return self.tmp(f"{a.c()} * {b.c()}")

    def add(self, a, b):
        if a.is_zero():
            return b
        if b.is_zero():
            return a
        if a.const is not None and b.const is not None:
            raise ValueError("constant folding beyond 0/+-1 not needed here")
        return self.tmp(f"{a.c()} + {b.c()}")

    def sub(self, a, b):
        if b.is_zero():
            return a
        if a.is_zero():
            return self.neg(b)
        if a.const is not None and b.const is not None:
            if a.const == b.const:
                return ZERO
            raise ValueError("unexpected constant difference")
        return self.tmp(f"{a.c()} - {b.c()}")

    def div(self, a, b):
        if a.is_zero():
            return ZERO
        return self.tmp(f"{a.c()} / {b.c()}")

    def acc(self, s, t):
        """s += t for a sum that started at 0.0."""
        if t.is_zero():
            return s
        if s.is_zero():
            return self.tmp(f"plus_zero({t.c()})")
        return self.add(s, t)


def inv4(gen, a):
    """types.rs:34-47 stand-in: the adjugate by 2x2 minors, the same sequence
    as inv4() in metric_fp64.cuh; returns (inverse entries, det)."""
    (a00, a01, a02, a03), (a10, a11, a12, a13), (a20, a21, a22, a23), (a30, a31, a32, a33) = a
    m, s_, n_ = gen.mul, gen.sub, gen.neg
    diff = s_
    s0 = diff(m(a00, a11), m(a10, a01))
    s1 = diff(m(a00, a12), m(a10, a02))
    s2 = diff(m(a00, a13), m(a10, a03))
    s3 = diff(m(a01, a12), m(a11, a02))
    s4 = diff(m(a01, a13), m(a11, a03))
    s5 = diff(m(a02, a13), m(a12, a03))
    c5 = diff(m(a22, a33), m(a32, a23))
    c4 = diff(m(a21, a33), m(a31, a23))
    c3 = diff(m(a21, a32), m(a31, a22))
    c2 = diff(m(a20, a33), m(a30, a23))
    c1 = diff(m(a20, a32), m(a30, a22))
    c0 = diff(m(a20, a31), m(a30, a21))
    A = gen.add
    det = A(s_(A(A(s_(m(s0, c5), m(s1, c4)), m(s2, c3)), m(s3, c2)), m(s4, c1)), m(s5, c0))
    if det.is_zero():
        raise ValueError("structurally singular metric")
    ident = gen.div(ONE, det)
    # write the 16 entries exactly as metric_fp64.cuh's inv4 does:
    out = [None] * 16
    out[0] = gen.mul(A(s_(m(a11, c5), m(a12, c4)), m(a13, c3)), ident)
    out[1] = gen.mul(s_(A(m(n_(a01), c5), m(a02, c4)), m(a03, c3)), ident)
    out[2] = gen.mul(A(s_(m(a31, s5), m(a32, s4)), m(a33, s3)), ident)
    out[3] = gen.mul(s_(A(m(n_(a21), s5), m(a22, s4)), m(a23, s3)), ident)
    out[4] = gen.mul(s_(A(m(n_(a10), c5), m(a12, c2)), m(a13, c1)), ident)
    out[5] = gen.mul(A(s_(m(a00, c5), m(a02, c2)), m(a03, c1)), ident)
    out[6] = gen.mul(s_(A(m(n_(a30), s5), m(a32, s2)), m(a33, s1)), ident)
    out[7] = gen.mul(A(s_(m(a20, s5), m(a22, s2)), m(a23, s1)), ident)
    out[8] = gen.mul(A(s_(m(a10, c4), m(a11, c2)), m(a13, c0)), ident)
    out[9] = gen.mul(s_(A(m(n_(a00), c4), m(a01, c2)), m(a03, c0)), ident)
    out[10] = gen.mul(A(s_(m(a30, s4), m(a31, s2)), m(a33, s0)), ident)
    out[11] = gen.mul(s_(A(m(n_(a20), s4), m(a21, s2)), m(a23, s0)), ident)
    out[12] = gen.mul(s_(A(m(n_(a10), c3), m(a11, c1)), m(a12, c0)), ident)
    out[13] = gen.mul(A(s_(m(a00, c3), m(a01, c1)), m(a02, c0)), ident)
    out[14] = gen.mul(s_(A(m(n_(a30), s3), m(a31, s1)), m(a32, s0)), ident)
    out[15] = gen.mul(A(s_(m(a20, s3), m(a21, s1)), m(a22, s0)), ident)
    return out, det


def christoffel(gen, g0, dgv):
    """metric/mod.rs:51-69 on symbolic ginv and dg; returns Gamma[64]."""
    ginv, det = inv4(gen, g0)
    gen.lines.append(f"  singular = ({det.c()}) == 0.0;")
    G = [None] * 64
    for mu in range(4):
        for al in range(4):
            for be in range(4):
                s = ZERO
                for sg in range(4):
                    br = gen.sub(gen.add(dgv[al][sg][be], dgv[be][sg][al]), dgv[sg][al][be])
                    s = gen.acc(s, gen.mul(ginv[4 * mu + sg], br))
                G[16 * mu + 4 * al + be] = ZERO if s.is_zero() else gen.tmp(f"0.5 * {s.c()}")
    return G


def rhs_terms(gen, G):
    """geodesic.rs:38-59: dp^mu = -sum_{a,b} Gamma^mu_ab p^a p^b, zero terms dropped."""
    lines = []
    for mu in range(4):
        sacc = ZERO
        for al in range(4):
            for be in range(4):
                gv = G[16 * mu + 4 * al + be]
                if gv.is_zero():
                    continue
                t = gen.mul(gen.mul(gv, V(expr=f"y[{4 + al}]")), V(expr=f"y[{4 + be}]"))
                sacc = gen.acc(sacc, t)
        lines.append(f"  k[{4 + mu}] = -({sacc.c()});" if not sacc.is_zero() else f"  k[{4 + mu}] = -0.0;")
    return lines


def metric_matrix(gen, spec, tag):
    """spec: 4x4 of 'zero', 'one', 'mone' or a runtime variable name."""
    out = []
    for i in range(4):
        row = []
        for j in range(4):
            v = spec[i][j]
            row.append({"zero": ZERO, "one": ONE, "mone": MONE}.get(v) or V(expr=f"{v}{tag}"))
        out.append(row)
    return out


def build(name, doc, spec, depends_on, evaluator):
    """spec: structure of g with runtime names; depends_on: axes g depends on;
    evaluator: C code computing the runtime names at point `xs` with suffix `tag`."""
    gen = Gen()
    body = []
    g0 = metric_matrix(gen, spec, "_c")
    body.append(evaluator("x", "_c"))
    dgv = [[[ZERO] * 4 for _ in range(4)] for _ in range(4)]
    for al in range(4):
        if al not in depends_on:
            continue  # g(x + h e_al) == g(x - h e_al) bit for bit: dg = (g - g)/two_h = +0
        body.append(f"  double xp{al}[4] = {{x[0], x[1], x[2], x[3]}};")
        body.append(f"  double xm{al}[4] = {{x[0], x[1], x[2], x[3]}};")
        body.append(f"  xp{al}[{al}] += FD_H;")
        body.append(f"  xm{al}[{al}] -= FD_H;")
        body.append(evaluator(f"xp{al}", f"_p{al}"))
        body.append(evaluator(f"xm{al}", f"_m{al}"))
        gp = metric_matrix(gen, spec, f"_p{al}")
        gm = metric_matrix(gen, spec, f"_m{al}")
        for mu in range(4):
            for nu in range(4):
                d = gen.sub(gp[mu][nu], gm[mu][nu])
                if d.const is not None:
                    dgv[al][mu][nu] = ZERO
                else:
                    dgv[al][mu][nu] = gen.div(d, V(expr="two_h"))
    n_dg = len(gen.lines)
    gen.lines = body + ["  const double two_h = 2.0 * FD_H;"] + gen.lines
    n_body = len(body)
    G = christoffel(gen, g0, dgv)
    calc = ["  const double two_h = 2.0 * FD_H;"] + gen.lines[n_body + 1:]
    assert len(calc) >= n_dg + 1
    nan_fill = ["  if (singular) {",
                "    const double nan = __longlong_as_double(0x7ff8000000000000LL);",
                "    for (int i = 0; i < 64; ++i) G[i] = nan;",
                "  }"]
    out = [f"// {doc}",
           f"__device__ __forceinline__ bool christoffel_{name}_sparse(const MetricDesc& M, const double x[4], "
           "double G[64]) {",
           "  bool singular;"]
    out += gen.lines
    for i, v in enumerate(G):
        out.append(f"  G[{i}] = {v.c()};")
    out += nan_fill
    out.append("  return !singular;")
    out.append("}")
    # The same Gamma from metric values evaluated elsewhere: gv holds, for the
    # tags _c, _p{a}, _m{a} (a over depends_on in order), the spec's runtime
    # names in order of first appearance. Same expressions, same bits.
    names = []
    for row in spec:
        for v in row:
            if v not in ("zero", "one", "mone") and v not in names:
                names.append(v)
    tags = ["_c"] + [f"_{pm}{a}" for a in depends_on for pm in ("p", "m")]
    unpack = []
    for ti, tag in enumerate(tags):
        for ni, nm in enumerate(names):
            unpack.append(f"  const double {nm}{tag} = gv[{ti * len(names) + ni}];")
    frm = [f"// {name}: Gamma from the metric values at the {len(tags)} finite-difference points (order above)",
           f"constexpr int {name.upper()}_VALUES = {len(names)};",
           f"__device__ __forceinline__ bool christoffel_{name}_from(const double* gv, double G[64]) {{",
           "  bool singular;"]
    frm += unpack + calc
    for i, v in enumerate(G):
        frm.append(f"  G[{i}] = {v.c()};")
    frm += nan_fill
    frm.append("  return !singular;")
    frm.append("}")
    # The RHS: same Gamma code, then the sums over the nonzero entries.
    n0 = len(gen.lines)
    rl = rhs_terms(gen, G)
    sums = gen.lines[n0:]
    rhs = [f"// geodesic.rs:38-59 right-hand side for {name}, Gamma as above",
           f"__device__ __forceinline__ bool rhs_{name}_sparse(const MetricDesc& M, const double y[8], "
           "double k[8]) {",
           "  const double* x = y;",
           "  bool singular;"]
    rhs += gen.lines[:n0] + sums
    rhs += ["  k[0] = y[4]; k[1] = y[5]; k[2] = y[6]; k[3] = y[7];"] + rl
    rhs += ["  return !singular;", "}"]
    return "\n".join(out) + "\n\n" + "\n".join(frm) + "\n\n" + "\n".join(rhs), gen


ALC_EVAL = """  double g00{t}, g01{t};
  alc_g00_g01(M, {x}, &g00{t}, &g01{t});"""
MT_EVAL = """  double g22{t}, g33{t};
  mt_g22_g33(M, {x}, &g22{t}, &g33{t});"""


ALC_SPEC = [["g00", "g01", "zero", "zero"], ["g01", "one", "zero", "zero"],
            ["zero", "zero", "one", "zero"], ["zero", "zero", "zero", "one"]]
MT_SPEC = [["mone", "zero", "zero", "zero"], ["zero", "one", "zero", "zero"],
           ["zero", "zero", "g22", "zero"], ["zero", "zero", "zero", "g33"]]
ALC_DEPENDS, MT_DEPENDS = (1, 2, 3), (1, 2)


def build_all():
    alc = build("alcubierre",
                "Alcubierre (alcubierre.rs:48-63): g depends on x^1..x^3 only; g_tt, g_tx, g_xt vary",
                ALC_SPEC, ALC_DEPENDS, lambda x, t: ALC_EVAL.format(x=x, t=t))
    mt = build("morris_thorne",
               "Morris-Thorne (morris_thorne.rs:22-36): g depends on l and theta; g_thth, g_phph vary",
               MT_SPEC, MT_DEPENDS, lambda x, t: MT_EVAL.format(x=x, t=t))
    return alc, mt


# Arithmetic of one metric evaluation at one point (alc_g00_g01, mt_g22_g33 in
# metric_fp64.cuh, which follow alcubierre.rs:33-63 and morris_thorne.rs:22-36),
# besides the calls counted on their own.
G_EVAL_FLOPS = {"alcubierre": 17, "morris_thorne": 5}
G_EVAL_CALLS = {"alcubierre": {"sqrt": 1, "tanh": 2}, "morris_thorne": {"sincos": 1}}
RK4_COMBINE_FLOPS = 104  # integrator.rs:16-40 on the 8 components: 3 stage points + the weighted sum


def op_counts():
    """Algorithmic FP64 work of one right-hand side and one RK4 step of the
    finite-difference fallback (metric/mod.rs:25-69, geodesic.rs:38-59) with
    the operations on structurally zero entries removed: the operations the
    generator emits (finite differences, inverse, contraction, the sums of the
    geodesic equation), plus the metric evaluations at the distinct
    finite-difference points (the centre and +-h along each axis g depends on;
    along the others the two evaluations are equal bit for bit and their
    difference is an exact zero)."""
    out = {}
    for (text, gen), name, dep in zip(build_all(), ("alcubierre", "morris_thorne"), (ALC_DEPENDS, MT_DEPENDS)):
        ops = {"mul": 0, "add": 0, "sub": 0, "div": 0}
        for line in gen.lines:
            m = re.match(r"\s*const double t\d+ = (.*);$", line)
            if not m:
                continue
            expr = m.group(1)
            for sym, key in ((" * ", "mul"), (" + ", "add"), (" - ", "sub"), (" / ", "div")):
                if sym in expr:
                    ops[key] += 1
                    break
        points = 1 + 2 * len(dep)
        calls = {k: v * points for k, v in G_EVAL_CALLS[name].items()}
        per_rhs = sum(ops.values()) + points * G_EVAL_FLOPS[name]
        out[name] = {"ops_per_rhs": ops, "metric_points_per_rhs": points,
                     "metric_eval_flops_per_rhs": points * G_EVAL_FLOPS[name],
                     "calls_per_rhs": calls, "flops_per_rhs": per_rhs,
                     "flops_per_step": 4 * per_rhs + RK4_COMBINE_FLOPS,
                     "calls_per_step": {k: 4 * v for k, v in calls.items()}}
    return out


def header_text():
    """The text of christoffel_sparse.cuh."""
    (alc, _), (mt, _) = build_all()
    header = """// GENERATED by gen_sparse_christoffel.py - do not edit by hand.
//
// Sparse FP64 Christoffel symbols, bit-identical (up to the sign of zero
// entries) to christoffel_generic<K> of metric_fp64.cuh, i.e. to the
// reference's finite-difference fallback (metric/mod.rs:25-69) with the
// adjugate inverse. Exactly-zero terms of the dense algorithm are dropped;
// everything else is evaluated in the dense algorithm's order.
#pragma once
"""
    return header + "\n" + alc + "\n\n" + mt + "\n"


def main():
    with open(os.path.join(HERE, "christoffel_sparse.cuh"), "w") as f:
        f.write(header_text())
    for name, c in op_counts().items():
        print(f"{name}: {c['ops_per_rhs']} per right-hand side, {c['flops_per_step']} flops per RK4 step")


if __name__ == "__main__":
    main()
