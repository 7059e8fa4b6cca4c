#!/usr/bin/env python3
"""Generates pairing_program.cuh: the phase tables of the warp-per-check pairing.

A 2-pair pairing check (Miller loop over precomputed lines, final
exponentiation) is a fixed sequence of Fp12 operations.  Each operation is
compiled here into a *program* of phases that one warp (32 lanes) runs over a
per-check array of Fp slots in shared memory:

  MUL phase : lane l computes slot[out] = slot[a] * slot[b]   (one Fp product)
  LIN phase : lane l computes slot[out] = sum_k +-slot[t_k]   (at most 6 terms)
  INV phase : lane 0 computes slot[out] = slot[a]^-1

Every lane runs the same instruction stream in a phase (only its table entry
differs), so the assembly of Karatsuba products costs a few modular additions
per lane instead of the divergent per-lane code of an Fp2-level team.

The Fp12 formulas are written once below over a symbolic Fp type whose
products become MUL nodes and whose additions stay linear forms until a
product or an output needs them.  The graph is scheduled greedily into
alternating LIN / MUL phases (at most 32 nodes each, longest path first),
temporaries get slots by liveness, and every program is checked numerically
against an independent schoolbook Fp12 (tower Fp2 = Fp[u]/(u^2+1),
Fp6 = Fp2[v]/(v^3 - (1+u)), Fp12 = Fp6[w]/(w^2 - v)) before it is emitted.

Formulas: Fp2/Fp6/Fp12 Karatsuba and the complex Fp12 squaring; the sparse
line value l(P) = A + (B xP) v + yP v w; Granger-Scott cyclotomic squaring
("Faster squaring in the cyclotomic subgroup of sixth degree extensions",
PKC 2010); Fp12 inverse through the Fp6 and Fp2 norms.

Usage: python gen_pairing_program.py [--check-only]
"""
import pathlib
import random
import sys

P = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB
LANES = 32
TMAX = 6          # terms per LIN entry
NONE = 0xFFFF

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
class Graph:
    def __init__(self):
        self.kind = []      # 'in', 'mul', 'lin', 'inv'
        self.args = []      # in: slot; mul: (a, b); lin: [(sign, node)]; inv: a
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

    def materialize(self, form):
        """Node holding the linear form {node: coef}."""
        form = {n: c for n, c in form.items() if c}
        if not form:
            return self.inp(ZERO_SLOT)
        if len(form) == 1:
            (n, c), = form.items()
            if c == 1:
                return n
        terms = []
        for n, c in sorted(form.items(), key=lambda x: (x[1] < 0, x[0])):
            terms += [(1 if c > 0 else -1, n)] * abs(c)
        while len(terms) > TMAX:  # split into a tree of LIN nodes
            head, terms = terms[:TMAX], terms[TMAX:]
            terms.append((1, self._lin(head)))
        return self._lin(terms)

    def _lin(self, terms):
        terms = sorted(terms, key=lambda t: (t[0] < 0, t[1]))
        return self._add("lin", terms, ("lin", tuple(terms)))

    def mul(self, fa, fb):
        a, b = self.materialize(fa), self.materialize(fb)
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
    """Results of Fp2 products are kept in slots of their own (as nodes): the
    sums built on them stay short, which shortens the assembly phases."""
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
        self.phases = []   # (type, [entry per lane])  type 0 LIN, 1 MUL, 2 INV; entry (out, op, args)
        self.ntmp = 0
        self.nmul = 0


def compile_program(name, builder):
    g = Graph()
    outs = builder(g)
    # output nodes: one LIN per output slot, built from the form (unshared)
    out_nodes = []
    for slot, v in outs:
        form = {n: c for n, c in v.f.items() if c}
        terms = []
        for n, c in sorted(form.items(), key=lambda x: (x[1] < 0, x[0])):
            terms += [(1 if c > 0 else -1, n)] * abs(c)
        if not terms:
            terms = [(1, g.inp(ZERO_SLOT))]
        while len(terms) > TMAX:
            head, terms = terms[:TMAX], terms[TMAX:]
            terms.append((1, g._lin(head)))
        g.kind.append("lin")
        g.args.append(sorted(terms, key=lambda t: (t[0] < 0, t[1])))
        out_nodes.append((len(g.kind) - 1, slot))
    out_of = {n: s for n, s in out_nodes}

    def deps(n):
        k, a = g.kind[n], g.args[n]
        if k == "in":
            return []
        if k == "mul":
            return list(a)
        if k == "inv":
            return [a]
        return [t[1] for t in a]

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
    prog = Program(name)
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
    prog.ntmp = ntmp
    for ptype, batch in plan:
        entries = []
        for n in batch:
            k, a = g.kind[n], g.args[n]
            if k == "mul":
                entries.append((slot[n], "mul", (slot[a[0]], slot[a[1]])))
                prog.nmul += 1
            elif k == "inv":
                entries.append((slot[n], "inv", (slot[a],)))
            else:
                entries.append((slot[n], "lin", tuple((sg, slot[t]) for sg, t in a)))
        prog.phases.append((ptype, entries))
    return prog


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


def simulate(prog, slots):
    s = dict(slots)
    for ptype, entries in prog.phases:
        res = []
        for out, op, args in entries:
            if op == "mul":
                res.append((out, s[args[0]] * s[args[1]] % P))
            elif op == "inv":
                res.append((out, pow(s[args[0]], P - 2, P)))
            else:
                res.append((out, sum(sg * s[t] for sg, t in args) % P))
        for out, v in res:
            s[out] = v
    return s


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


def emit(progs):
    nslot = TMP_BASE + max(p.ntmp for p in progs)
    lines = ["// GENERATED by gen_pairing_program.py -- do not edit by hand.",
             "// Phase tables of the warp-per-check pairing (see pairing_team.cuh).",
             "#pragma once", "#include <stdint.h>", "",
             "#define PP_LANES %d" % LANES, "#define PP_NONE 0x%04x" % NONE,
             "#define PP_SLOTS %d" % nslot, "#define PP_LINE_BASE %d" % LINE_BASE,
             "#define PP_PT_BASE %d" % PT_BASE, "#define PP_GAMMA_BASE %d" % GAMMA_BASE,
             "#define PP_ZERO_SLOT %d" % ZERO_SLOT,
             "#define PP_REG(r) (12 * (r))",
             "enum { PP_REG_F, PP_REG_T, PP_REG_A, PP_REG_X, PP_REG_R, PP_REG_U };",
             "enum { PP_LIN = 0, PP_MUL = 1, PP_INV = 2 };", ""]
    lines.append("enum {" + ", ".join("PP_" + n for n in ORDER) + ", PP_NPROG };")
    first, types, ents = [], [], []
    for p in progs:
        first.append(len(types))
        for ptype, entries in p.phases:
            types.append(ptype)
            row = []
            # every lane of a LIN phase runs the phase's largest term count;
            # shorter sums are padded with the zero slot
            width = max((len(a) for _, op, a in entries if op == "lin"), default=0)
            for l in range(LANES):
                u = [NONE, ptype << 8 | width, 0, 0, 0, 0, 0, 0]
                if l < len(entries):
                    out, op, args = entries[l]
                    u[0] = out
                    if op == "lin":
                        padded = list(args) + [(1, ZERO_SLOT)] * (width - len(args))
                        for t, (sg, sl) in enumerate(padded):
                            assert sl < 0x8000
                            u[2 + t] = sl | (0x8000 if sg < 0 else 0)
                    else:
                        for t, sl in enumerate(args):
                            u[2 + t] = sl
                row.append("{0x%08x, 0x%08x, 0x%08x, 0x%08x}" % tuple(u[2 * k] | (u[2 * k + 1] << 16)
                                                                     for k in range(4)))
            ents.append("  " + ", ".join(row) + ",")
    first.append(len(types))
    lines.append("#define PP_NPHASE %d" % len(types))
    lines.append("__device__ const uint16_t PP_PROG_FIRST[PP_NPROG + 1] = {" + ", ".join(map(str, first)) + "};")
    lines.append("// entry per (phase, lane): u16 out (PP_NONE: idle lane), u16 phase type << 8 | term count")
    lines.append("// (LIN: the same count on every lane of the phase, short sums padded with the zero slot),")
    lines.append("// then u16 x 6 terms (LIN; bit 15: subtract) or operand slots (MUL: a, b; INV: a)")
    lines.append("__device__ const uint4 PP_ENTRY[PP_NPHASE * PP_LANES] = {")
    lines += ents
    lines.append("};")
    summary = ["// %-11s %3d phases (%s), %3d products, %3d temporaries" %
               (p.name, len(p.phases), "".join("LMI"[t] for t, _ in p.phases), p.nmul, p.ntmp) for p in progs]
    return "\n".join(lines[:4] + summary + lines[4:]) + "\n"


def main():
    rng = random.Random(20240601)
    progs = []
    for name in ORDER:
        p = compile_program(name, PROGRAMS[name])
        check(p, rng)
        progs.append(p)
    text = emit(progs)
    if "--check-only" not in sys.argv:
        out = pathlib.Path(__file__).resolve().parent / "pairing_program.cuh"
        out.write_text(text)
        print("wrote", out, "phases:", sum(len(p.phases) for p in progs))


if __name__ == "__main__":
    main()
