"""Generate curve_constants.cuh: BLS12-381 constants in Montgomery form
(R = 2^384 for Fp) for the device code.

Every constant is computed here from the curve parameters:
  * p, r, z (BLS parameter, z = -0xd201000000010000), the generators of G1/G2;
  * beta: the cube root of unity in Fp with [z^2](x, y) = (beta*x, -y) on G1
    (the GLV endomorphism) -- checked on the G1 generator;
  * Fp12 Frobenius coefficients gamma_k = xi^(k(p-1)/6), xi = 1 + u;
  * the SSWU 11-isogeny E' -> E used by hash_to_curve (RFC 9380 suite
    BLS12381G1_XMD:SHA-256_SSWU_RO_).  Its kernel polynomial is the product of
    the five linear factors of the 11-division polynomial of E' over Fp (the
    unique Fp-rational 11-torsion subgroup); Velu's formulas give the isogeny,
    which is composed with the isomorphism (x, y) -> (u^2 x, u^3 y) onto
    y^2 = x^3 + 4.  Of the six u with u^6 = 4 / B_codomain, the one whose
    hash_to_curve output matches the CFRG draft's first BBS message generator
    (Q1 below, a published test vector) is kept.

Run:  python gen_curve_constants.py            (uses the stored kernel and u)
      python gen_curve_constants.py --derive   (re-derives them, ~10 s)
"""
import hashlib
import pathlib
import random
import sys

P = int("1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab", 16)
R = int("73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001", 16)
Z_ABS = 0xD201000000010000
G1X = int("17f1d3a73197d7942695638c4fa9ac0fc3688c4f9774b905a14e3a3f171bac586c55e83ff97a1aeffb3af00adb22c6bb", 16)
G1Y = int("08b3f481e3aaa0f1a09e30ed741d8ae4fcf5e095d5d00af600db18cb2c04b3edd03cc744a2888ae40caa232946c5e7e1", 16)
G2X0 = int("024aa2b2f08f0a91260805272dc51051c6e47ad4fa403b02b4510b647ae3d1770bac0326a805bbefd48056c8c121bdb8", 16)
G2X1 = int("13e02b6052719f607dacd3a088274f65596bd0d09920b61ab5da61bbdc7f5049334cf11213945d57e5ac7d055d042b7e", 16)
G2Y0 = int("0ce5d527727d6e118cc9cdc6da2e351aadfd9baa8cbdd3a76d429a695160d12c923ac9cc3baca289e193548608b82801", 16)
G2Y1 = int("0606c4a02ea734cc32acd2b02bc28b99cb3e287e85a763af267492ab572e99ab3f370d275cec1da1aaa9075ff05f79be", 16)
# BBS ciphersuite base point P1 (ciphersuites.rs:78) and the first message generator Q1.
P1_HEX = "a8ce256102840821a3e94ea9025e4662b205762f9776b3a766c872b948f1fd225e7c59698588e70d11406d161b4e28c9"
Q1_HEX = "a9ec65b70a7fbe40c874c9eb041c2cb0a7af36ccec1bea48fa2ba4c2eb67ef7f9ecb17ed27d38d27cdeddff44c8137be"
SSWU_A = int("144698a3b8e9433d693a02c96d4982b0ea985383ee66a8d8e8981aefd881ac98936f8da0e0f97f5cf428082d584c1d", 16)
SSWU_B = int("12e2908d11688030018b12e8753eee3b2016c1f0f24f4070a0b9c14fcef35ef55a23215a316ceaa5d1cc48e98e172be0", 16)
SSWU_Z = 11
# Stored results of --derive (kernel polynomial low->high, monic, and u).
ISO_KERNEL = [
    0x133341fb0962a34cb0504a9c4fada0a5090d38679b4c040d5d1c3afb023a3409fcc0815fea66d8b02bbef9c8b5a66e07,
    0x264908af037bcede00d054cf5d4775e83eb6cf63c76b969f8ed174fb59fcff78d201f46f6cfc4ed6552e59ce75177b0,
    0x1335c502c1f54c49aceea65e87fd7203ba0f626f305fc0cfd606a5dae9f3c8e81a4b3b69600129fabd307c69bf319d39,
    0x94440f65f408a6e930e16e3e92dd17bf60d6e9679a8d3d58593de55ac23703042d609537eb3549aac234d896ca82944,
    0x4afe09d5cf4956a23b6b71f59d2b3407b415a774b7be81bbb6fa99cbc798e0ac98ba725a5bc328016b1c268b4766e85,
    1,
]
ISO_U = 0x17a3e1bda8a2d1a38a19241a0ea1e2f25b552d6197903f96bae690ef6be6b1381be22e8a72a9745cd7a1ffffffffb26d


def inv(a):
    return pow(a, P - 2, P)


def sqrt(a):
    s = pow(a, (P + 1) // 4, P)
    return s if s * s % P == a % P else None


# ---------------- polynomial helpers over Fp (coefficients low -> high)
def trim(a):
    while a and a[-1] == 0:
        a.pop()
    return a


def padd(a, b):
    n = max(len(a), len(b))
    return trim([((a[i] if i < len(a) else 0) + (b[i] if i < len(b) else 0)) % P for i in range(n)])


def psub(a, b):
    n = max(len(a), len(b))
    return trim([((a[i] if i < len(a) else 0) - (b[i] if i < len(b) else 0)) % P for i in range(n)])


def pmul(a, b):
    if not a or not b:
        return []
    r = [0] * (len(a) + len(b) - 1)
    for i, x in enumerate(a):
        if x:
            for j, y in enumerate(b):
                r[i + j] += x * y
    return trim([c % P for c in r])


def pscale(a, c):
    return trim([x * c % P for x in a])


def pdivmod(a, b):
    a = a[:]
    q = [0] * max(0, len(a) - len(b) + 1)
    ib = inv(b[-1])
    while len(a) >= len(b) and a:
        c = a[-1] * ib % P
        d = len(a) - len(b)
        q[d] = c
        for i, y in enumerate(b):
            a[i + d] = (a[i + d] - c * y) % P
        trim(a)
    return trim(q), a


def pmod(a, b):
    return pdivmod(a, b)[1]


def pgcd(a, b):
    while b:
        a, b = b, pmod(a, b)
    return pscale(a, inv(a[-1])) if a else a


def pderiv(a):
    return trim([(i * a[i]) % P for i in range(1, len(a))])


def ppowmod(base, e, m):
    res = [1]
    base = pmod(base, m)
    while e:
        if e & 1:
            res = pmod(pmul(res, base), m)
        base = pmod(pmul(base, base), m)
        e >>= 1
    return res


def peval(poly, x):
    r = 0
    for c in reversed(poly):
        r = (r * x + c) % P
    return r


# ---------------- affine group law (None = infinity)
def ec_add(p1, p2, a=0):
    if p1 is None:
        return p2
    if p2 is None:
        return p1
    (x1, y1), (x2, y2) = p1, p2
    if x1 == x2:
        if (y1 + y2) % P == 0:
            return None
        lam = (3 * x1 * x1 + a) * inv(2 * y1) % P
    else:
        lam = (y2 - y1) * inv(x2 - x1) % P
    x3 = (lam * lam - x1 - x2) % P
    return (x3, (lam * (x1 - x3) - y1) % P)


def ec_mul(k, pt, a=0):
    acc = None
    while k:
        if k & 1:
            acc = ec_add(acc, pt, a)
        pt = ec_add(pt, pt, a)
        k >>= 1
    return acc


def velu_maps(D, a, b):
    """x-map N/D^2 and y-map y*Yn/D^3 of the normalised isogeny with kernel polynomial D."""
    Dp = pderiv(D)
    Rv = pmod(pmul([2 * a % P, 0, 6], Dp), D)
    Ru = pmod(pmul([4 * b % P, 4 * a % P, 0, 4], Dp), D)
    D2 = pmul(D, D)
    N = padd(padd(pmul([0, 1], D2), pmul(Rv, D)), psub(pmul(Ru, Dp), pmul(pderiv(Ru), D)))
    Yn = psub(pmul(pderiv(N), D), pscale(pmul(N, Dp), 2))
    return N, D2, Yn, pmul(D2, D)


def derive_kernel():
    a, b = SSWU_A, SSWU_B
    F = [4 * b % P, 4 * a % P, 0, 4]
    cache = {0: [], 1: [1], 2: [1],
             3: trim([(-a * a) % P, 12 * b % P, 6 * a % P, 0, 3]),
             4: pscale(trim([(-8 * b * b - a ** 3) % P, (-4 * a * b) % P, (-5 * a * a) % P,
                             20 * b % P, 5 * a % P, 0, 1]), 2)}

    def f(n):  # psi_n for odd n, psi_n / 2y for even n
        if n in cache:
            return cache[n]
        m = n // 2
        if n % 2:
            t1 = pmul(f(m + 2), pmul(f(m), pmul(f(m), f(m))))
            t2 = pmul(f(m - 1), pmul(f(m + 1), pmul(f(m + 1), f(m + 1))))
            res = psub(pmul(pmul(F, F), t1), t2) if m % 2 == 0 else psub(t1, pmul(pmul(F, F), t2))
        else:
            res = pmul(f(m), psub(pmul(f(m + 2), pmul(f(m - 1), f(m - 1))),
                                  pmul(f(m - 2), pmul(f(m + 1), f(m + 1)))))
        cache[n] = res
        return res

    f11 = f(11)
    f11 = pscale(f11, inv(f11[-1]))
    h = ppowmod([0, 1], P, f11)
    return pgcd(psub(h, [0, 1]), f11)  # product of the linear factors


def expand_xmd(msg, dst, n):
    ell = (n + 31) // 32
    dstp = dst + bytes([len(dst)])
    b0 = hashlib.sha256(bytes(64) + msg + n.to_bytes(2, "big") + b"\0" + dstp).digest()
    bs = [hashlib.sha256(b0 + b"\1" + dstp).digest()]
    for i in range(2, ell + 1):
        bs.append(hashlib.sha256(bytes(x ^ y for x, y in zip(b0, bs[-1])) + bytes([i]) + dstp).digest())
    return b"".join(bs)[:n]


def sswu(u):
    A, B, Z = SSWU_A, SSWU_B, SSWU_Z
    tv1 = (Z * Z * pow(u, 4, P) + Z * u * u) % P
    x1 = B * inv(Z * A) % P if tv1 == 0 else (-B * inv(A)) * (1 + inv(tv1)) % P
    y = sqrt((x1 ** 3 + A * x1 + B) % P)
    x = x1
    if y is None:
        x = Z * u * u * x1 % P
        y = sqrt((x ** 3 + A * x + B) % P)
    if (u % 2) != (y % 2):
        y = (-y) % P
    return x, y


def compress(pt):
    x, y = pt
    bb = bytearray(x.to_bytes(48, "big"))
    bb[0] |= 0x80 | (0x20 if y > (P - 1) // 2 else 0)
    return bytes(bb).hex()


def hash_to_curve(msg, dst, maps, u):
    N, D2, Yn, D3 = maps
    ub = expand_xmd(msg, dst, 128)
    acc = None
    for k in range(2):
        x, y = sswu(int.from_bytes(ub[64 * k:64 * k + 64], "big") % P)
        X = u * u * peval(N, x) * inv(peval(D2, x)) % P
        Y = pow(u, 3, P) * y * peval(Yn, x) * inv(peval(D3, x)) % P
        acc = ec_add(acc, (X, Y))
    return ec_mul(0xD201000000010001, acc)


def first_generator_seed():
    api = b"BBS_BLS12381G1_XMD:SHA-256_SSWU_RO_H2G_HM2S_"
    seed_dst = api + b"SIG_GENERATOR_SEED_"
    v = expand_xmd(api + b"MESSAGE_GENERATOR_SEED", seed_dst, 48)
    return expand_xmd(v + (1).to_bytes(8, "big"), seed_dst, 48), api + b"SIG_GENERATOR_DST_"


def derive_isogeny():
    D = derive_kernel()
    assert len(D) == 6, "expected a degree-5 rational kernel"
    maps = velu_maps(D, SSWU_A, SSWU_B)
    # codomain B of the Velu curve: B2 = b - 7 * sum(10x^3 + 6ax + 4b) over kernel x-coords
    roots_ps = newton_sums(D, 3)
    w = (10 * roots_ps[3] + 6 * SSWU_A * roots_ps[1] + 20 * SSWU_B) % P
    B2 = (SSWU_B - 7 * w) % P
    target = (4 * inv(B2)) % P
    cands = sixth_roots(target)
    msg, dst = first_generator_seed()
    good = [u for u in cands if compress(hash_to_curve(msg, dst, maps, u)) == Q1_HEX]
    assert len(good) == 1
    return D, good[0]


def newton_sums(D, k):
    d = len(D) - 1
    e = [1] + [((-1) ** i) * D[d - i] % P for i in range(1, d + 1)]
    ps = [0] * (k + 1)
    for m in range(1, k + 1):
        s = sum(((-1) ** (i - 1)) * e[i] * ps[m - i] for i in range(1, min(m, d + 1)) if i < m)
        if m <= d:
            s += ((-1) ** (m - 1)) * m * e[m]
        ps[m] = s % P
    return ps


def sixth_roots(t):
    # p = 3 mod 4 and p = 1 mod 3: find all x with x^6 = t by brute-forcing a cube root then square roots
    from sympy.ntheory.residue_ntheory import nthroot_mod
    return nthroot_mod(t, 6, P, all_roots=True)


# ---------------- emission helpers
def limbs32(x, n=12):
    return [(x >> (32 * i)) & 0xFFFFFFFF for i in range(n)]


def mont(x):
    return (x << 384) % P


def fp_init(x):
    return "{{" + ", ".join(f"0x{w:08x}u" for w in limbs32(mont(x % P))) + "}}"


def main():
    global ISO_KERNEL, ISO_U
    if "--derive" in sys.argv:
        D, u = derive_isogeny()
        assert D == ISO_KERNEL and u == ISO_U, "re-derived isogeny differs from the stored one"
        print("re-derived isogeny matches the stored kernel polynomial and u")
    maps = velu_maps(ISO_KERNEL, SSWU_A, SSWU_B)
    u = ISO_U
    xnum = pscale(maps[0], u * u % P)
    xden = maps[1]
    ynum = pscale(maps[2], pow(u, 3, P))
    yden = maps[3]
    msg, dst = first_generator_seed()
    assert compress(hash_to_curve(msg, dst, maps, u)) == Q1_HEX
    # GLV endomorphism
    lam = Z_ABS * Z_ABS
    s = sqrt(P - 3)
    betas = [(-1 + s) * inv(2) % P, (-1 - s) * inv(2) % P]
    zz = ec_mul(lam, (G1X, G1Y))
    beta = [b for b in betas if (b * G1X % P, (-G1Y) % P) == zz][0]
    # Frobenius gammas for Fp12 = Fp2[w]/(w^6 - xi)
    def f2mul(a, b):
        return ((a[0] * b[0] - a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)

    def f2pow(a, e):
        r = (1, 0)
        while e:
            if e & 1:
                r = f2mul(r, a)
            a = f2mul(a, a)
            e >>= 1
        return r

    g = f2pow((1, 1), (P - 1) // 6)
    gammas = [(1, 0)]
    for _ in range(5):
        gammas.append(f2mul(gammas[-1], g))
    p1 = bytes.fromhex(P1_HEX)
    lines = [
        "// GENERATED by gen_curve_constants.py -- do not edit by hand.",
        "// BLS12-381 constants in Montgomery form (R = 2^384) as fp initialisers.",
        "#pragma once",
        "",
        f"#define C_FP_ONE {fp_init(1)}",
        f"#define C_FP_TWO {fp_init(2)}",
        f"#define C_FP_THREE {fp_init(3)}",
        f"#define C_FP_FOUR {fp_init(4)}",
        f"#define C_FP_INV2 {fp_init(inv(2))}",
        f"#define C_G1_GEN_X {fp_init(G1X)}",
        f"#define C_G1_GEN_Y {fp_init(G1Y)}",
        f"#define C_G2_GEN_X0 {fp_init(G2X0)}",
        f"#define C_G2_GEN_X1 {fp_init(G2X1)}",
        f"#define C_G2_GEN_Y0 {fp_init(G2Y0)}",
        f"#define C_G2_GEN_Y1 {fp_init(G2Y1)}",
        f"// beta: [z^2](x, y) = (beta x, -y) on G1, z^2 = 0x{lam:x}",
        f"#define C_GLV_BETA {fp_init(beta)}",
        f"#define C_GLV_LAMBDA_LO 0x{lam & ((1 << 64) - 1):016x}ull",
        f"#define C_GLV_LAMBDA_HI 0x{lam >> 64:016x}ull",
        f"#define C_SSWU_A {fp_init(SSWU_A)}",
        f"#define C_SSWU_B {fp_init(SSWU_B)}",
        f"#define C_SSWU_Z {fp_init(SSWU_Z)}",
        f"#define C_SSWU_MINUS_B_OVER_A {fp_init((-SSWU_B) * inv(SSWU_A))}",
        f"#define C_SSWU_B_OVER_ZA {fp_init(SSWU_B * inv(SSWU_Z * SSWU_A))}",
        f"#define C_ISO_XNUM_LEN {len(xnum)}",
        f"#define C_ISO_XDEN_LEN {len(xden)}",
        f"#define C_ISO_YNUM_LEN {len(ynum)}",
        f"#define C_ISO_YDEN_LEN {len(yden)}",
        "#define C_ISO_XNUM {" + ", ".join(fp_init(c) for c in xnum) + "}",
        "#define C_ISO_XDEN {" + ", ".join(fp_init(c) for c in xden) + "}",
        "#define C_ISO_YNUM {" + ", ".join(fp_init(c) for c in ynum) + "}",
        "#define C_ISO_YDEN {" + ", ".join(fp_init(c) for c in yden) + "}",
        "// Frobenius: gamma_k = xi^(k(p-1)/6) as (c0, c1) pairs, k = 0..5",
        "#define C_FROB_GAMMA {" + ", ".join("{" + fp_init(a) + ", " + fp_init(b) + "}" for a, b in gammas) + "}",
        "#define C_P1_COMPRESSED {" + ", ".join(f"0x{b:02x}" for b in p1) + "}",
        "",
    ]
    dst_path = pathlib.Path(__file__).with_name("curve_constants.cuh")
    dst_path.write_text("\n".join(lines))
    print("wrote", dst_path)


if __name__ == "__main__":
    main()
