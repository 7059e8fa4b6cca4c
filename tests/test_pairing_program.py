"""The phase tables of the warp-per-check pairing (pairing_program.cuh), for
one-warp and two-warp teams, decoded the way pp::run in pairing_team.cuh
decodes them, against the independent schoolbook Fp12 of gen_pairing_program.py.

The weighted sums are emulated limb for limb: 64-bit accumulators per limb,
the single-precision quotient estimate taken from the top two accumulators
before any carry, one signed carry pass and two conditional subtractions, so a
table entry or a bound that the device arithmetic would get wrong fails here.
"""
import importlib.util
import pathlib
import random
import re

import numpy as np
import pytest

CSRC = pathlib.Path(__file__).resolve().parents[1] / "cubbs-cred_gb300" / "csrc"


@pytest.fixture(scope="module")
def gen():
    spec = importlib.util.spec_from_file_location("gen_pairing_program", CSRC / "gen_pairing_program.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module", params=[("", 32), ("_W", 64)], ids=["one-warp", "two-warp"])
def table(request):
    """The phase table of one team width: (first phase per program, words, slots, lanes)."""
    sfx, lanes = request.param
    txt = (CSRC / "pairing_program.cuh").read_text()
    assert int(re.search(r"#define PP_LANES%s (\d+)" % sfx, txt).group(1)) == lanes
    first = [int(x) for x in re.search(r"PP_PROG_FIRST%s\[PP_NPROG \+ 1\] = \{([^}]*)\}" % re.escape(sfx),
                                       txt).group(1).split(",")]
    start = txt.index("PP_ENTRY%s[PP_NPHASE%s * PP_LANES%s * 2] = {" % (sfx, sfx, sfx))
    body = txt[start:txt.index("};", start)]
    words = [int(x, 16) for x in re.findall(r"0x([0-9a-f]{8})", body)]
    nslot = int(re.search(r"#define PP_SLOTS (\d+)", txt).group(1))
    assert len(words) == first[-1] * lanes * 8
    return first, words, nslot, lanes


P = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB
PL = [(P >> (32 * j)) & 0xFFFFFFFF for j in range(12)]
INV_PTOP = np.float32(1.0) / np.float32(436277739.0)


def wsum_device(vals_coefs):
    """The device reduction of sum k x (x in [0, p), |k| <= 64)."""
    acc = [0] * 12
    for x, k in vals_coefs:
        v, m = (P - x, -k) if k < 0 else (x, k)
        for j in range(12):
            acc[j] += ((v >> (32 * j)) & 0xFFFFFFFF) * m
    assert max(acc) < 1 << 42
    top = acc[11] + (acc[10] >> 32)
    q = int(np.float32(top) * INV_PTOP)
    q = q - 1 if q else 0
    c, r = 0, 0
    for j in range(12):
        c += acc[j] - q * PL[j]
        assert -(1 << 63) <= c < 1 << 63
        r |= (c & 0xFFFFFFFF) << (32 * j)
        c >>= 32
    assert c == 0 and 0 <= r < 4 * P
    if r >= 2 * P:
        r -= 2 * P
    if r >= P:
        r -= P
    return r


def _coef(v):
    k = (v >> 9) & 0x7F
    return k - 128 if k & 0x40 else k


def run_program(table, s, prog):
    first, words, _, lanes = table
    s = dict(s)
    for ph in range(first[prog], first[prog + 1]):
        res = []
        types = set()
        for lane in range(lanes):
            w = words[(ph * lanes + lane) * 8:(ph * lanes + lane) * 8 + 8]
            u = [(w[i // 2] >> (16 * (i % 2))) & 0xFFFF for i in range(16)]
            out, tw = u[0], u[1]
            types.add(tw)
            if out == 0xFFFF:
                continue
            typ, na, nb = tw >> 12, tw & 15, (tw >> 4) & 15
            lo, hi = u[2:16], u[9:16]
            terms = lambda ts, n: [(s[v & 0x1FF], _coef(v)) for v in ts[:n]]
            if typ == 1:
                x = s[lo[0] & 0x1FF] if tw & 0x100 else wsum_device(terms(lo, na))
                y = s[hi[0] & 0x1FF] if tw & 0x200 else wsum_device(terms(hi, nb))
                r = x * y % P
            elif typ == 0:
                if tw & 0x100:  # plain sum: +-1 coefficients, bit 15 = subtract, at most 6 terms
                    assert na <= 6
                    tot = sum((P - s[v & 0x1FF]) if v & 0x8000 else s[v & 0x1FF] for v in lo[:na])
                    assert all(abs(_coef(v)) == 1 for v in lo[:na]) and tot < 8 * P
                    r = tot % P
                else:
                    r = wsum_device(terms(lo, na))
            else:
                assert typ == 2 and lane == 0
                r = pow(s[lo[0] & 0x1FF], P - 2, P)
            res.append((out, r))
        assert len(types) == 1, "type word differs between the lanes of a phase"
        for out, r in res:
            s[out] = r
    return s


def test_every_program_matches_schoolbook(gen, table):
    rng = random.Random(20250101)
    nslot = table[2]
    for prog, name in enumerate(gen.ORDER):
        s = gen.random_slots(rng, cyclo_regs=(gen.REG_R,) if name == "CYCLO_R" else ())
        for i in range(gen.TMP_BASE, nslot):  # temporaries hold junk on entry
            s[i] = rng.randrange(P)
        got = run_program(table, s, prog)
        r, want = gen.expected(name, s)
        assert gen.to_w(got, r) == want, name
        for q in range(6):
            if q != r:
                assert gen.to_w(got, q) == gen.to_w(s, q), (name, q)


def test_weighted_sum_reduction_bounds():
    rng = random.Random(7)
    edge = [0, 1, P - 1, (1 << 352) - 1, P - (1 << 320), ((1 << 320) - 1) % P]
    for _ in range(3000):
        n = rng.randrange(1, 15)
        xs = [rng.choice(edge + [rng.randrange(P)]) for _ in range(n)]
        ks = [rng.choice([-64, -63, 63, -1, 1, 2, -3, rng.randrange(-64, 64)]) for _ in range(n)]
        assert wsum_device(list(zip(xs, ks))) == sum(k * x for x, k in zip(xs, ks)) % P
    # the largest sums the encoding allows
    for k in (63, -64):
        assert wsum_device([(P - 1, k)] * 14) == (14 * k * (P - 1)) % P
