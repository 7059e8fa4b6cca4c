#!/usr/bin/env python3
"""Generates pairing_program.cuh: the phase tables of the warp-per-check pairing.

A 2-pair pairing check (Miller loop over precomputed lines, final
exponentiation) is a fixed sequence of Fp12 operations.  Each operation is
compiled here into a *program* of phases that a team of lanes (one warp of 32,
or two warps of 64) runs over a per-check array of Fp slots in shared memory:

  MUL phase : lane l computes slot[out] = (sum_i k_i slot[a_i]) * (sum_j k_j slot[b_j])
              (one Fp product of two short weighted sums, at most 7 terms each)
  LIN phase : lane l computes slot[out] = sum_i k_i slot[t_i]   (at most 14 terms)
  INV phase : lane 0 computes slot[out] = slot[a]^-1

The coefficients k are small signed integers (|k| < 64).  Every lane runs the
same instruction stream in a phase (only its table entry differs), so the
assembly of Karatsuba products costs a few multiply-adds per lane instead of
the divergent per-lane code of an Fp2-level team.

The Fp12 formulas are written once below over a symbolic Fp type whose
products become MUL nodes and whose additions stay weighted linear forms until
a product or an output needs them.  A form of at most KMUL terms is summed by
the product's own lane; a longer one becomes a LIN node.  A LIN node whose
only use is inside another sum is folded into it while the sum stays within
its width.  The graph is scheduled greedily into LIN / MUL phases (at most one
node per lane of the team, longest path first), temporaries get slots by liveness, and every
program is checked numerically against an independent schoolbook Fp12 (tower
Fp2 = Fp[u]/(u^2+1), Fp6 = Fp2[v]/(v^3 - (1+u)), Fp12 = Fp6[w]/(w^2 - v))
before it is emitted.  Each program is compiled under a few settings (LIN
width, product-operand width, whether Fp2 product results get slots of their
own) and the one with the lowest modelled cycle count is kept; the model's
per-phase costs were measured on the device for this kernel.

Formulas: Fp2/Fp6/Fp12 Karatsuba and the complex Fp12 squaring; the sparse
line value l(P) = A + (B xP) v + yP v w; Granger-Scott cyclotomic squaring
("Faster squaring in the cyclotomic subgroup of sixth degree extensions",
PKC 2010); Fp12 inverse through the Fp6 and Fp2 norms.

Usage: python gen_pairing_program.py [--check-only]
"""
import itertools
import pathlib
import random
import sys

P = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB
LANES = 32
NONE = 0xFFFF
SLOT_BITS = 9     # term = slot | (coefficient & 0x7f) << 9
COEF_MAX = 63
WLIN_MAX = 14     # terms per LIN entry
KMUL_MAX = 7      # terms per product operand
UNIT_MAX = 6      # LIN phases whose coefficients are all +-1 and at most this wide use the plain sum

# settings of one compilation (set by compile_program); with "expand", a
# coefficient k becomes |k| repeated terms of coefficient +-1, so the sums can
# run as plain LIN phases
CFG = {"wlin": 6, "kmul": 1, "mat": True, "expand": False}

# ----------------------------------------------------------------------------- slot map
# Six Fp12 registers of 12 slots each; register r, Fp2 coefficient k (0..5 =
# c0.c0, c0.c1, c0.c2, c1.c0, c1.c1, c1.c2), component j (0 = c0, 1 = c1):
# slot 12 r + 2 k + j.
REG_F, REG_T, REG_A, REG_X, REG_R, REG_U = range(6)
REG_NAMES = ["F", "T", "A", "X", "R", "U"]
LINE_BASE = 72    # pair p (0, 1): A.c0, A.c1, B.c0, B.c1 at LINE_BASE + 4 p + (0..3)
PT_BASE = 80      # pair p: xP, yP at PT_BASE + 2 p + (0, 1)
GAMMA_BASE = 84   # Frobenius gammas g[1..5] (Fp2) at GAMMA_BASE + 2 (k - 1) + j
ZERO_SLOT = 94
TMP_BASE = 96


def reg_slot(r, k, j):
    return 12 * r + 2 * k + j


# ----------------------------------------------------------------------------- graph
def _terms(form):
    """Canonical term tuple ((coef, node), ...) of a form {node: coef}."""
    t = sorted(((c, n) for n, c in form.items() if c), key=lambda t: (t[1], t[0]))
    if CFG["expand"]:
        t = [(1 if c > 0 else -1, n) for c, n in t for _ in range(abs(c))]
    return tuple(t)


class Graph:
    def __init__(self):
        self.kind = []      # 'in', 'mul', 'lin', 'inv'
        self.args = []      # in: slot; mul: (terms_a, terms_b); lin: terms; inv: node
        self.key = {}

    def _add(self, kind, args, key=None):
        if key is not None and key in self.key:
            return self.key[key]
        self.kind.append(kind)
        self.args.append(args)
        n = len(self.kind) - 1
        if key is not None:
            self.key[key] = n
        return n

    def inp(self, slot):
        return self._add("in", slot, ("in", slot))

    def lin(self, terms, width):
        """LIN node of the weighted terms, split into a tree of at most `width` terms each."""
        terms = list(terms)
        while len(terms) > width:
            head, terms = tuple(terms[:width]), terms[width:]
            terms.append((1, self._add("lin", head, ("lin", head))))
        terms = tuple(sorted(terms, key=lambda t: (t[1], t[0])))
        return self._add("lin", terms, ("lin", terms))

    def materialize(self, form):
        """Node holding the linear form {node: coef}."""
        t = _terms(form)
        if not t:
            return self.inp(ZERO_SLOT)
        if len(t) == 1 and t[0][0] == 1:
            return t[0][1]
        return self.lin(t, CFG["wlin"])

    def operand(self, form):
        t = _terms(form)
        if not t:
            return ((1, self.inp(ZERO_SLOT)),)
        if len(t) <= CFG["kmul"]:
            return t
        return ((1, self.materialize(form)),)

    def mul(self, fa, fb):
        a, b = self.operand(fa), self.operand(fb)
        a, b = min(a, b), max(a, b)
        return self._add("mul", (a, b), ("mul", a, b))

    def inv(self, fa):
        a = self.materialize(fa)
        return self._add("inv", a, ("inv", a))


class S:
    """Symbolic Fp value: a linear form over graph nodes."""

    def __init__(self, g, form):
        self.g, self.f = g, form

    @staticmethod
    def of(g, node):
        return S(g, {node: 1})

    def __add__(self, o):
        f = dict(self.f)
        for n, c in o.f.items():
            f[n] = f.get(n, 0) + c
        return S(self.g, {n: c for n, c in f.items() if c})

    def __neg__(self):
        return S(self.g, {n: -c for n, c in self.f.items()})

    def __sub__(self, o):
        return self + (-o)

    def scale(self, k):
        return S(self.g, {n: k * c for n, c in self.f.items()})

    def __mul__(self, o):
        return S.of(self.g, self.g.mul(self.f, o.f))

    def inv(self):
        return S.of(self.g, self.g.inv(self.f))


def _mul_s(a, b):
    """Product of two symbolic values; a zero operand gives zero without a node."""
    if not a.f or not b.f:
        return S(a.g, {})
    return a * b


# ----------------------------------------------------------------------------- tower over a base type
# The same classes run over S (to build programs) and over N (numbers mod p,
# to check them).  `mul` below is Karatsuba at every level.
class N:
    def __init__(self, v):
        self.v = v % P

    def __add__(self, o):
        return N(self.v + o.v)

    def __sub__(self, o):
        return N(self.v - o.v)

    def __neg__(self):
        return N(-self.v)

    def scale(self, k):
        return N(k * self.v)

    def __mul__(self, o):
        return N(self.v * o.v)

    def inv(self):
        return N(pow(self.v, P - 2, P))


def bmul(a, b):
    return _mul_s(a, b) if isinstance(a, S) else a * b


def mat(x):
    """With CFG["mat"], results of Fp2 products get slots of their own (as
    nodes), so the sums built on them stay short; without it they stay forms
    and fold into the sums and operands that use them."""
    if not CFG["mat"]:
        return x
    return S.of(x.g, x.g.materialize(x.f)) if isinstance(x, S) and x.f else x


class F2:
    def __init__(self, c0, c1):
        self.c0, self.c1 = c0, c1

    def __add__(self, o):
        return F2(self.c0 + o.c0, self.c1 + o.c1)

    def __sub__(self, o):
        return F2(self.c0 - o.c0, self.c1 - o.c1)

    def __neg__(self):
        return F2(-self.c0, -self.c1)

    def scale(self, k):
        return F2(self.c0.scale(k), self.c1.scale(k))

    def conj(self):
        return F2(self.c0, -self.c1)

    def mul_xi(self):  # (1 + u)(c0 + c1 u)
        return F2(self.c0 - self.c1, self.c0 + self.c1)

    def mul_fp(self, s):
        return F2(bmul(self.c0, s), bmul(self.c1, s))

    def __mul__(self, o):
        t0, t1 = bmul(self.c0, o.c0), bmul(self.c1, o.c1)
        t2 = bmul(self.c0 + self.c1, o.c0 + o.c1)
        return F2(mat(t0 - t1), mat(t2 - t0 - t1))

    def sqr(self):
        return F2(mat(bmul(self.c0 + self.c1, self.c0 - self.c1)), mat(bmul(self.c0, self.c1).scale(2)))


class F6:
    def __init__(self, c0, c1, c2):
        self.c = [c0, c1, c2]

    def __add__(self, o):
        return F6(*[a + b for a, b in zip(self.c, o.c)])

    def __sub__(self, o):
        return F6(*[a - b for a, b in zip(self.c, o.c)])

    def __neg__(self):
        return F6(*[-a for a in self.c])

    def scale(self, k):
        return F6(*[a.scale(k) for a in self.c])

    def mul_v(self):
        return F6(self.c[2].mul_xi(), self.c[0], self.c[1])

    def __mul__(self, o):
        a0, a1, a2 = self.c
        b0, b1, b2 = o.c
        p0, p1, p2 = a0 * b0, a1 * b1, a2 * b2
        p3, p4, p5 = (a1 + a2) * (b1 + b2), (a0 + a1) * (b0 + b1), (a0 + a2) * (b0 + b2)
        return F6(p0 + (p3 - p1 - p2).mul_xi(), p4 - p0 - p1 + p2.mul_xi(), p5 - p0 - p2 + p1)

    def mul_f2(self, s):
        return F6(*[a * s for a in self.c])


class F12:
    def __init__(self, c0, c1):
        self.c0, self.c1 = c0, c1

    def coeffs(self):
        """Fp2 coefficients in slot order c0.c0, c0.c1, c0.c2, c1.c0, c1.c1, c1.c2."""
        return self.c0.c + self.c1.c

    @staticmethod
    def from_coeffs(k):
        return F12(F6(*k[:3]), F6(*k[3:]))

    def conj(self):
        return F12(self.c0, -self.c1)

    def __mul__(self, o):
        t0, t1 = self.c0 * o.c0, self.c1 * o.c1
        return F12(t0 + t1.mul_v(), (self.c0 + self.c1) * (o.c0 + o.c1) - t0 - t1)

    def sqr(self):
        a0, a1 = self.c0, self.c1
        ab = a0 * a1
        t = (a0 + a1) * (a0 + a1.mul_v())
        return F12(t - ab - ab.mul_v(), ab.scale(2))

    def cyclo_sqr(self):
        """Granger-Scott squaring of an element of the cyclotomic subgroup."""
        S_ = self.coeffs()
        pa, pb = [0, 3, 1], [4, 2, 5]
        Z = []
        for g in range(3):
            x, y = S_[pa[g]], S_[pb[g]]
            Z += [x.sqr(), y.sqr(), (x + y).sqr()]
        out = [None] * 6

        def three_minus(t, v):  # 3 t - 2 v
            return (t - v).scale(2) + t

        def three_plus(t, v):   # 3 t + 2 v
            return (t + v).scale(2) + t
        out[0] = three_minus(Z[1].mul_xi() + Z[0], S_[0])
        out[4] = three_plus(Z[2] - Z[0] - Z[1], S_[4])
        out[1] = three_minus(Z[4].mul_xi() + Z[3], S_[1])
        out[5] = three_plus(Z[5] - Z[3] - Z[4], S_[5])
        out[3] = three_plus((Z[8] - Z[6] - Z[7]).mul_xi(), S_[3])
        out[2] = three_minus(Z[7].mul_xi() + Z[6], S_[2])
        return F12.from_coeffs(out)

    def frob(self, gammas):
        """x -> x^p; gammas[e] = xi^(e (p-1)/6) multiplies the coefficient of w^e."""
        wpow = [0, 2, 4, 1, 3, 5]
        out = []
        for k, c in enumerate(self.coeffs()):
            v = c.conj()
            out.append(v if k == 0 else v * gammas[wpow[k]])
        return F12.from_coeffs(out)

    def inv(self):
        c0, c1 = self.c0, self.c1
        D = c0 * c0 - (c1 * c1).mul_v()
        D0, D1, D2 = D.c
        t0 = D0.sqr() - (D1 * D2).mul_xi()
        t1 = D2.sqr().mul_xi() - D0 * D1
        t2 = D1.sqr() - D0 * D2
        d = D0 * t0 + (D2 * t1 + D1 * t2).mul_xi()
        nrm = bmul(d.c0, d.c0) + bmul(d.c1, d.c1)
        ni = nrm.inv()
        dinv = F2(bmul(d.c0, ni), -bmul(d.c1, ni))
        Dinv = F6(t0 * dinv, t1 * dinv, t2 * dinv)
        return F12(c0 * Dinv, -(c1 * Dinv))


def line_f12(A, Bx, yP, zero):
    """l(P) = A + (B xP) v + yP v w."""
    return F12(F6(A, Bx, F2(zero, zero)), F6(F2(zero, zero), F2(yP, zero), F2(zero, zero)))


# ----------------------------------------------------------------------------- program definitions
def sym_reg(g, r, conj=False):
    k = [F2(S.of(g, g.inp(reg_slot(r, c, 0))), S.of(g, g.inp(reg_slot(r, c, 1)))) for c in range(6)]
    f = F12.from_coeffs(k)
    return f.conj() if conj else f


def sym_gammas(g):
    return {e: F2(S.of(g, g.inp(GAMMA_BASE + 2 * (e - 1))), S.of(g, g.inp(GAMMA_BASE + 2 * (e - 1) + 1)))
            for e in range(1, 6)}


def sym_line(g, p):
    b = LINE_BASE + 4 * p
    A = F2(S.of(g, g.inp(b)), S.of(g, g.inp(b + 1)))
    B = F2(S.of(g, g.inp(b + 2)), S.of(g, g.inp(b + 3)))
    xP, yP = S.of(g, g.inp(PT_BASE + 2 * p)), S.of(g, g.inp(PT_BASE + 2 * p + 1))
    zero = S(g, {})
    return line_f12(A, B.mul_fp(xP), yP, zero)


def reg_out(r, f):
    out = []
    for c, v in enumerate(f.coeffs()):
        out += [(reg_slot(r, c, 0), v.c0), (reg_slot(r, c, 1), v.c1)]
    return out


def prog_dbl(g):
    f = sym_reg(g, REG_F)
    lam = sym_line(g, 0) * sym_line(g, 1)
    return reg_out(REG_F, f.sqr() * lam)


def prog_add(g):
    return reg_out(REG_F, sym_reg(g, REG_F) * (sym_line(g, 0) * sym_line(g, 1)))


def prog_dbl1(g):
    return reg_out(REG_F, sym_reg(g, REG_F).sqr() * sym_line(g, 0))


def prog_add1(g):
    return reg_out(REG_F, sym_reg(g, REG_F) * sym_line(g, 0))


PROGRAMS = {
    "DBL": prog_dbl,
    "ADD": prog_add,
    # one pair's Miller loop (a warp per pair; the warps' values are multiplied after)
    "DBL1": prog_dbl1,
    "ADD1": prog_add1,
    "MUL_F_F_X": lambda g: reg_out(REG_F, sym_reg(g, REG_F) * sym_reg(g, REG_X)),
    "CONJ_F": lambda g: reg_out(REG_F, sym_reg(g, REG_F, conj=True)),
    "INV_U_F": lambda g: reg_out(REG_U, sym_reg(g, REG_F).inv()),
    "EASY1_T": lambda g: reg_out(REG_T, sym_reg(g, REG_F, conj=True) * sym_reg(g, REG_U)),
    "EASY2_T": lambda g: reg_out(REG_T, sym_reg(g, REG_T).frob(sym_gammas(g)).frob(sym_gammas(g)) *
                                 sym_reg(g, REG_T)),
    "COPY_R_T": lambda g: reg_out(REG_R, sym_reg(g, REG_T)),
    "COPY_R_A": lambda g: reg_out(REG_R, sym_reg(g, REG_A)),
    "COPY_R_X": lambda g: reg_out(REG_R, sym_reg(g, REG_X)),
    "CYCLO_R": lambda g: reg_out(REG_R, sym_reg(g, REG_R).cyclo_sqr()),
    "MUL_R_R_T": lambda g: reg_out(REG_R, sym_reg(g, REG_R) * sym_reg(g, REG_T)),
    "MUL_R_R_A": lambda g: reg_out(REG_R, sym_reg(g, REG_R) * sym_reg(g, REG_A)),
    "MUL_R_R_X": lambda g: reg_out(REG_R, sym_reg(g, REG_R) * sym_reg(g, REG_X)),
    "S1_A": lambda g: reg_out(REG_A, sym_reg(g, REG_R, conj=True) * sym_reg(g, REG_T, conj=True)),
    "S2_A": lambda g: reg_out(REG_A, sym_reg(g, REG_R, conj=True) * sym_reg(g, REG_A, conj=True)),
    "S3_A": lambda g: reg_out(REG_A, sym_reg(g, REG_R, conj=True) * sym_reg(g, REG_A).frob(sym_gammas(g))),
    "S4_X": lambda g: reg_out(REG_X, sym_reg(g, REG_R, conj=True)),
    "S5_R": lambda g: reg_out(REG_R, sym_reg(g, REG_R, conj=True) *
                              sym_reg(g, REG_A).frob(sym_gammas(g)).frob(sym_gammas(g))),
    "MUL_R_R_CA": lambda g: reg_out(REG_R, sym_reg(g, REG_R) * sym_reg(g, REG_A, conj=True)),
}


# ----------------------------------------------------------------------------- compile
class Program:
    def __init__(self, name):
        self.name = name
        # (type, [entry per lane]); type 0 LIN, 1 MUL, 2 INV
        # entry: (out, 'lin', terms) | (out, 'mul', (terms_a, terms_b)) | (out, 'inv', terms)
        # with terms ((coef, slot), ...)
        self.phases = []
        self.ntmp = 0
        self.nmul = 0
        self.cfg = None


def _fold(g, terms, width):
    """Replaces LIN-node terms by their own terms while the sum stays within `width`."""
    form = {}
    for c, n in terms:
        form[n] = form.get(n, 0) + c
    changed = True
    while changed:
        changed = False
        for n in sorted(form, reverse=True):
            if g.kind[n] != "lin":
                continue
            cand = dict(form)
            c = cand.pop(n)
            for c2, m in g.args[n]:
                cand[m] = cand.get(m, 0) + c * c2
            cand = {m: v for m, v in cand.items() if v}
            if 0 < len(_terms(cand)) <= width and all(abs(v) <= COEF_MAX for v in cand.values()):
                form, changed = cand, True
                break
    return _terms(form)


def compile_program(name, builder, cfg):
    CFG.update(cfg)
    g = Graph()
    outs = builder(g)
    out_nodes = []  # one LIN per output slot (unshared)
    for slot, v in outs:
        t = _terms(v.f) or ((1, g.inp(ZERO_SLOT)),)
        if len(t) > CFG["wlin"]:
            t = g.args[g.lin(t, CFG["wlin"])]
        g.kind.append("lin")
        g.args.append(t)
        out_nodes.append((len(g.kind) - 1, slot))
    for n in range(len(g.kind)):  # nodes are in topological order
        if g.kind[n] == "mul":
            a, b = g.args[n]
            g.args[n] = (_fold(g, a, CFG["kmul"]), _fold(g, b, CFG["kmul"]))
        elif g.kind[n] == "lin":
            g.args[n] = _fold(g, g.args[n], CFG["wlin"])
    for n in range(len(g.kind)):
        for c, _ in (g.args[n][0] + g.args[n][1] if g.kind[n] == "mul" else
                     g.args[n] if g.kind[n] == "lin" else ()):
            assert abs(c) <= COEF_MAX, (name, c)
    out_of = {n: s for n, s in out_nodes}

    def deps(n):
        k, a = g.kind[n], g.args[n]
        if k == "in":
            return []
        if k == "mul":
            return [m for _, m in a[0] + a[1]]
        if k == "inv":
            return [a]
        return [m for _, m in a]

    # reachable set
    need, stack = set(), [n for n, _ in out_nodes]
    while stack:
        n = stack.pop()
        if n in need:
            continue
        need.add(n)
        stack += deps(n)
    users = {n: [] for n in need}
    for n in need:
        for d in deps(n):
            users[d].append(n)
    height = {}

    def h(n):
        if n not in height:
            height[n] = 1 + max([h(u) for u in users[n]], default=0)
        return height[n]
    for n in need:
        h(n)
    done = {n for n in need if g.kind[n] == "in"}
    todo = need - done
    phase_of = {}
    plan = []
    while todo:
        ready = [n for n in todo if all(d in done for d in deps(n))]
        non_out = [n for n in ready if n not in out_of]
        if not (todo - set(out_of)):
            batch, ptype = sorted(ready), 0
            assert len(batch) == len(todo) <= LANES, (name, len(batch))
        else:
            lin = [n for n in non_out if g.kind[n] == "lin"]
            mul = [n for n in non_out if g.kind[n] == "mul"]
            inv = [n for n in non_out if g.kind[n] == "inv"]
            if lin:
                batch, ptype = sorted(lin, key=lambda n: -height[n])[:LANES], 0
            elif mul:
                batch, ptype = sorted(mul, key=lambda n: -height[n])[:LANES], 1
            else:
                assert inv, name
                batch, ptype = inv[:1], 2
        for n in batch:
            phase_of[n] = len(plan)
        plan.append((ptype, batch))
        done |= set(batch)
        todo -= set(batch)
    # slots: inputs fixed, outputs fixed, temporaries by liveness
    last_use = {}
    for n in need:
        for u in users[n]:
            last_use[n] = max(last_use.get(n, -1), phase_of[u])
    slot = {n: g.args[n] for n in need if g.kind[n] == "in"}
    slot.update(out_of)
    free, busy, ntmp = [], [], 0
    for k, (ptype, batch) in enumerate(plan):
        still = []
        for (end, s) in busy:
            if end <= k:
                free.append(s)
            else:
                still.append((end, s))
        busy = still
        free.sort()
        for n in batch:
            if n in out_of:
                continue
            if free:
                s = free.pop(0)
            else:
                s = TMP_BASE + ntmp
                ntmp += 1
            slot[n] = s
            busy.append((last_use[n], s))
    prog = Program(name)
    prog.ntmp = ntmp
    prog.cfg = dict(cfg)
    st = lambda terms: tuple((c, slot[m]) for c, m in terms)
    for ptype, batch in plan:
        entries = []
        for n in batch:
            k, a = g.kind[n], g.args[n]
            if k == "mul":
                entries.append((slot[n], "mul", (st(a[0]), st(a[1]))))
                prog.nmul += 1
            elif k == "inv":
                entries.append((slot[n], "inv", ((1, slot[a]),)))
            else:
                entries.append((slot[n], "lin", st(a)))
        prog.phases.append((ptype, entries))
    return prog


# ----------------------------------------------------------------------------- cost model
# Cycles of one warp, fitted to the measured cycles of every program on GB300
# (within about 2 percent): an Fp product 2860; a weighted product operand
# 403 + 191 per term; a LIN phase with coefficients +-1 452 + 189 per term, a
# weighted one 814 + 192 per term; the inverse ~79k; 150 per program run.
def _plain(terms):
    return len(terms) == 1 and terms[0][0] == 1


def _unit(entries):
    return all(abs(c) == 1 for _, _, t in entries for c, _ in t) and max(len(t) for _, _, t in entries) <= UNIT_MAX


def phase_cost(ptype, entries):
    if ptype == 2:
        return 79000
    if ptype == 1:
        c = 2860
        for side in (0, 1):
            if not all(_plain(e[2][side]) for e in entries):
                c += 403 + 191 * max(len(e[2][side]) for e in entries)
        return c
    w = max(len(t) for _, _, t in entries)
    return 452 + 189 * w if _unit(entries) else 814 + 192 * w


def program_cost(prog):
    return 150 + sum(phase_cost(t, e) for t, e in prog.phases)


SETTINGS = [{"wlin": w, "kmul": k, "mat": m, "expand": x}
            for w, k, m, x in itertools.product([4, 6, 8, 10, 12, 14], [1, 2, 3, 4, 6, 7], [True, False],
                                                [False, True])]


def best_program(name, rng):
    best = None
    for cfg in SETTINGS:
        try:
            p = compile_program(name, PROGRAMS[name], cfg)
        except AssertionError:
            continue
        if best is None or program_cost(p) < program_cost(best):
            best = p
    check(best, rng)
    return best


# ----------------------------------------------------------------------------- independent check
# Schoolbook Fp12 as polynomials of degree < 6 in w over Fp2 (w^6 = xi = 1 + u);
# slot-order coefficient k multiplies w^WPOW[k].
WPOW = [0, 2, 4, 1, 3, 5]


def f2m(a, b):
    return ((a[0] * b[0] - a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)


def f2a(a, b):
    return ((a[0] + b[0]) % P, (a[1] + b[1]) % P)


def wmul(x, y):
    r = [(0, 0)] * 11
    for i in range(6):
        for j in range(6):
            r[i + j] = f2a(r[i + j], f2m(x[i], y[j]))
    for k in range(10, 5, -1):  # w^k = xi w^(k-6)
        r[k - 6] = f2a(r[k - 6], f2m(r[k], (1, 1)))
    return r[:6]


def wpow(x, e):
    r = [(1, 0)] + [(0, 0)] * 5
    for bit in bin(e)[2:]:
        r = wmul(r, r)
        if bit == "1":
            r = wmul(r, x)
    return r


def to_w(slots, r):
    w = [None] * 6
    for k in range(6):
        w[WPOW[k]] = (slots[reg_slot(r, k, 0)], slots[reg_slot(r, k, 1)])
    return w


def wconj(x):
    return [c if e % 2 == 0 else ((-c[0]) % P, (-c[1]) % P) for e, c in enumerate(x)]


def gammas():
    xi = [(1, 1)] + [(0, 0)] * 5
    out = {}
    for e in range(1, 6):
        g = [(1, 0)] + [(0, 0)] * 5
        base = (1, 1)
        # xi^(e (p - 1) / 6) in Fp2
        val = (1, 0)
        ex = e * (P - 1) // 6
        b = base
        while ex:
            if ex & 1:
                val = f2m(val, b)
            b = f2m(b, b)
            ex >>= 1
        out[e] = val
    return out


def random_slots(rng, cyclo_regs=()):
    s = {i: rng.randrange(P) for i in range(TMP_BASE)}
    s[ZERO_SLOT] = 0
    gm = gammas()
    for e in range(1, 6):
        s[GAMMA_BASE + 2 * (e - 1)], s[GAMMA_BASE + 2 * (e - 1) + 1] = gm[e]
    for r in cyclo_regs:  # put a cyclotomic element (f^((p^6-1)(p^2+1))) into register r
        f = to_w(s, r)
        g = wmul(wconj(f), wpow(f, P ** 12 - 2))
        g = wmul(wpow(g, P * P), g)
        for k in range(6):
            s[reg_slot(r, k, 0)], s[reg_slot(r, k, 1)] = g[WPOW[k]]
    return s


def expected(name, s):
    F, T, A, X, R, U = (to_w(s, r) for r in range(6))
    frob = lambda x: wpow(x, P)
    def line(p):
        b = LINE_BASE + 4 * p
        xP, yP = s[PT_BASE + 2 * p], s[PT_BASE + 2 * p + 1]
        l = [(0, 0)] * 6
        l[0] = (s[b], s[b + 1])
        l[2] = f2m((s[b + 2], s[b + 3]), (xP, 0))
        l[3] = (yP, 0)
        return l
    lam = wmul(line(0), line(1))
    table = {
        "DBL": (REG_F, lambda: wmul(wmul(F, F), lam)),
        "ADD": (REG_F, lambda: wmul(F, lam)),
        "DBL1": (REG_F, lambda: wmul(wmul(F, F), line(0))),
        "ADD1": (REG_F, lambda: wmul(F, line(0))),
        "MUL_F_F_X": (REG_F, lambda: wmul(F, X)),
        "CONJ_F": (REG_F, lambda: wconj(F)),
        "INV_U_F": (REG_U, lambda: wpow(F, P ** 12 - 2)),
        "EASY1_T": (REG_T, lambda: wmul(wconj(F), U)),
        "EASY2_T": (REG_T, lambda: wmul(frob(frob(T)), T)),
        "COPY_R_T": (REG_R, lambda: T), "COPY_R_A": (REG_R, lambda: A), "COPY_R_X": (REG_R, lambda: X),
        "CYCLO_R": (REG_R, lambda: wmul(R, R)),
        "MUL_R_R_T": (REG_R, lambda: wmul(R, T)), "MUL_R_R_A": (REG_R, lambda: wmul(R, A)),
        "MUL_R_R_X": (REG_R, lambda: wmul(R, X)),
        "S1_A": (REG_A, lambda: wmul(wconj(R), wconj(T))),
        "S2_A": (REG_A, lambda: wmul(wconj(R), wconj(A))),
        "S3_A": (REG_A, lambda: wmul(wconj(R), frob(A))),
        "S4_X": (REG_X, lambda: wconj(R)),
        "S5_R": (REG_R, lambda: wmul(wconj(R), frob(frob(A)))),
        "MUL_R_R_CA": (REG_R, lambda: wmul(R, wconj(A))),
    }
    r, fn = table[name]
    return r, fn()


def simulate(prog, slots):
    s = dict(slots)
    wsum = lambda terms: sum(c * s[t] for c, t in terms)
    for ptype, entries in prog.phases:
        res = []
        for out, op, args in entries:
            if op == "mul":
                res.append((out, wsum(args[0]) * wsum(args[1]) % P))
            elif op == "inv":
                res.append((out, pow(wsum(args), P - 2, P)))
            else:
                res.append((out, wsum(args) % P))
        for out, v in res:
            s[out] = v
    return s


def check(prog, rng, trials=2):
    for _ in range(trials):
        s = random_slots(rng, cyclo_regs=(REG_R,) if prog.name == "CYCLO_R" else ())
        got = simulate(prog, s)
        r, want = expected(prog.name, s)
        assert to_w(got, r) == want, prog.name
        # registers other than the output are untouched
        for q in range(6):
            if q != r:
                assert to_w(got, q) == to_w(s, q), (prog.name, q)


# ----------------------------------------------------------------------------- emission
ORDER = list(PROGRAMS)
T_LIN, T_MUL, T_INV = 0, 1, 2
F_UNIT_OR_PLAIN_A, F_PLAIN_B = 0x100, 0x200


def _term(c, sl):
    assert 0 <= sl < (1 << SLOT_BITS) and -64 <= c <= COEF_MAX
    return sl | ((c & 0x7F) << SLOT_BITS)


def phase_words(ptype, entries, lanes):
    """16 u16 words per lane: out, type word, terms 0..6 (LIN terms / operand a),
    terms 7..13 (LIN terms / operand b)."""
    pad = lambda terms, n, unit: list(terms) + [(1 if unit else 0, ZERO_SLOT)] * (n - len(terms))
    rows = []
    if ptype == 1:
        plain = [all(_plain(e[2][side]) for e in entries) for side in (0, 1)]
        width = [1 if plain[side] else max(len(e[2][side]) for e in entries) for side in (0, 1)]
        assert max(width) <= KMUL_MAX
        tw = T_MUL << 12 | width[1] << 4 | width[0] | (F_UNIT_OR_PLAIN_A if plain[0] else 0) | \
            (F_PLAIN_B if plain[1] else 0)
    elif ptype == 2:
        tw = T_INV << 12 | 1
    else:
        width = max(len(t) for _, _, t in entries)
        assert width <= WLIN_MAX
        unit = _unit(entries)
        tw = T_LIN << 12 | width | (F_UNIT_OR_PLAIN_A if unit else 0)
    for l in range(lanes):
        u = [NONE, tw] + [_term(0, ZERO_SLOT)] * 14
        if l < len(entries):
            out, op, args = entries[l]
            u[0] = out
            if op == "mul":
                for side in (0, 1):
                    for t, (c, sl) in enumerate(pad(args[side], width[side], False)):
                        u[2 + 7 * side + t] = _term(c, sl)
            else:
                for t, (c, sl) in enumerate(pad(args, width if op == "lin" else 1, op == "lin" and unit)):
                    u[2 + t] = _term(c, sl)
        rows.append(u)
    return rows


def _table_lines(progs, lanes, sfx):
    """PP_PROG_FIRST<sfx> and PP_ENTRY<sfx> for one team width."""
    first, ents, nph = [], [], 0
    for p in progs:
        first.append(nph)
        for ptype, entries in p.phases:
            assert len(entries) <= lanes
            nph += 1
            row = []
            for u in phase_words(ptype, entries, lanes):
                w = [u[2 * k] | (u[2 * k + 1] << 16) for k in range(8)]
                row.append("{0x%08x, 0x%08x, 0x%08x, 0x%08x}, {0x%08x, 0x%08x, 0x%08x, 0x%08x}" % tuple(w))
            ents.append("  " + ", ".join(row) + ",")
    first.append(nph)
    lines = ["#define PP_NPHASE%s %d" % (sfx, nph),
             "__device__ const uint16_t PP_PROG_FIRST%s[PP_NPROG + 1] = {%s};" % (sfx, ", ".join(map(str, first))),
             "__device__ const uint4 PP_ENTRY%s[PP_NPHASE%s * PP_LANES%s * 2] = {" % (sfx, sfx, sfx)]
    return lines + ents + ["};"]


def _summary(progs, lanes):
    out = ["// %d lanes:" % lanes]
    for p in progs:
        desc = ""
        for t, e in p.phases:
            if t == 1:
                desc += "M"
            elif t == 2:
                desc += "I"
            else:
                desc += "L" if _unit(e) else "W"
        out.append("// %-11s %3d phases (%s), %3d products, %3d temporaries, ~%d cycles" %
                   (p.name, len(p.phases), desc, p.nmul, p.ntmp, program_cost(p)))
    return out


def emit(sets):
    """sets: [(lanes, programs)], the one-warp team first."""
    nslot = TMP_BASE + max(p.ntmp for _, progs in sets for p in progs)
    assert nslot <= 1 << SLOT_BITS
    lines = ["// GENERATED by gen_pairing_program.py -- do not edit by hand.",
             "// Phase tables of the warp-per-check pairing (see pairing_team.cuh).",
             "#pragma once", "#include <stdint.h>", "",
             "#define PP_LANES %d" % sets[0][0], "#define PP_LANES_W %d" % sets[1][0],
             "#define PP_NONE 0x%04x" % NONE,
             "#define PP_SLOTS %d" % nslot, "#define PP_LINE_BASE %d" % LINE_BASE,
             "#define PP_PT_BASE %d" % PT_BASE, "#define PP_GAMMA_BASE %d" % GAMMA_BASE,
             "#define PP_ZERO_SLOT %d" % ZERO_SLOT,
             "#define PP_REG(r) (12 * (r))",
             "enum { PP_REG_F, PP_REG_T, PP_REG_A, PP_REG_X, PP_REG_R, PP_REG_U };",
             "enum { PP_LIN = %d, PP_MUL = %d, PP_INV = %d };" % (T_LIN, T_MUL, T_INV),
             "#define PP_F_UNIT 0x%03x    // LIN: coefficients +-1, at most %d terms" % (F_UNIT_OR_PLAIN_A, UNIT_MAX),
             "#define PP_F_PLAIN_A 0x%03x // MUL: operand a is one slot with coefficient 1" % F_UNIT_OR_PLAIN_A,
             "#define PP_F_PLAIN_B 0x%03x // MUL: operand b likewise" % F_PLAIN_B, ""]
    lines.append("enum {" + ", ".join("PP_" + n for n in ORDER) + ", PP_NPROG };")
    lines.append("// Two uint4 per (phase, lane), as 16 u16: out slot (PP_NONE: idle lane); type << 12 |")
    lines.append("// flags | nb << 4 | na (LIN: na = term count, the same on every lane of the phase);")
    lines.append("// terms 0..6 (LIN terms, MUL operand a); terms 7..13 (LIN terms, MUL operand b).")
    lines.append("// A term is slot | (signed 7-bit coefficient) << 9; short sums are padded with the zero slot.")
    lines.append("// PP_*: one-warp teams (PP_LANES lanes); PP_*_W: two-warp teams (PP_LANES_W lanes).")
    lines += _table_lines(sets[0][1], sets[0][0], "")
    lines += _table_lines(sets[1][1], sets[1][0], "_W")
    summary = []
    for lanes, progs in sets:
        summary += _summary(progs, lanes)
    return "\n".join(lines[:4] + summary + lines[4:]) + "\n"


def compile_all(lanes, rng):
    """Every program for a team of `lanes` lanes (phases of at most that many entries)."""
    global LANES
    LANES = lanes
    return [best_program(name, rng) for name in ORDER]


def main():
    rng = random.Random(20240601)
    sets = [(32, compile_all(32, rng)), (64, compile_all(64, rng))]
    text = emit(sets)
    if "--check-only" not in sys.argv:
        out = pathlib.Path(__file__).resolve().parent / "pairing_program.cuh"
        out.write_text(text)
        print("wrote", out, "phases:", [sum(len(p.phases) for p in progs) for _, progs in sets])
    for lanes, progs in sets:
        for p in progs:
            print("%2d lanes %-11s %3d phases ~%6d cycles  %s" % (lanes, p.name, len(p.phases), program_cost(p), p.cfg))


if __name__ == "__main__":
    main()
