"""GPU parity for the primitive ABI entry points (MSMs, G1 add, prepare-B,
T2-prepare, pairing equality) against the oracle and the native KATs."""
import pytest

from helpers import R_MOD, drbg, keypair, scalar

h = bytes.fromhex
pytestmark = pytest.mark.gpu


def rand_points(oracle, seed, n):
    p1, _ = oracle.generators(1)
    return [oracle.g1_mul(p1, scalar(seed, b"pt", i)) for i in range(n)]


def rand_scalars(seed, label, n):
    return [scalar(seed, label, i) for i in range(n)]


def test_prepare_b_kat_via_msm(gpu, golden):
    k = golden["prepare_b_kat"]
    (code, out), = gpu.g1_msm_batch([([h(p) for p in k["msm_points"]], [h(s) for s in k["msm_scalars"]])])
    assert code == 0 and out.hex() == k["expected_b"]
    rows = gpu.g1_msm_common_points([h(p) for p in k["msm_points"]], [[h(s) for s in k["msm_scalars"]]])
    assert rows[0][0] == 0 and rows[0][2].hex() == k["expected_b"]
    assert rows[0][1] == 2  # resident generator tables (route 2)


def test_prepare_b_kat(gpu, golden):
    k = golden["prepare_b_kat"]
    (code, b), = gpu.prepare_b_batch([(h(k["public_key"]), h(k["header"]), [h(s) for s in k["message_scalars"]])])
    assert code == 0 and b.hex() == k["expected_b"]


@pytest.mark.parametrize("terms", [1, 2, 3, 17, 64])
def test_g1_msm_batch(gpu, oracle, terms):
    seed = b"msm-%d" % terms
    msms = []
    for i in range(5):
        pts = rand_points(oracle, seed + bytes([i]), terms)
        scs = rand_scalars(seed + bytes([i]), b"s", terms)
        msms.append((pts, scs))
    got = gpu.g1_msm_batch(msms)
    for (pts, scs), (code, out) in zip(msms, got):
        assert code == 0 and out == oracle.g1_msm(pts, scs)


def test_g1_msm_edge_scalars(gpu, oracle):
    p = rand_points(oracle, b"edge", 3)
    zero, one = bytes(32), (1).to_bytes(32, "big")
    rm1 = (R_MOD - 1).to_bytes(32, "big")
    cases = [([p[0]], [zero]), ([p[0]], [one]), ([p[0]], [rm1]), ([p[0], p[0]], [one, rm1]),
             ([p[0], p[0]], [one, one]), ([], [])]
    got = gpu.g1_msm_batch(cases)
    for (pts, scs), (code, out) in zip(cases, got):
        assert code == 0 and out == oracle.g1_msm(pts, scs)
    # non-canonical scalar -> item error
    code, _ = gpu.g1_msm_batch([([p[0]], [R_MOD.to_bytes(32, "big")])])[0]
    assert code == gpu.ERR_INVALID_INPUT


@pytest.mark.parametrize("K", [12, 102])
def test_common_points_generators(gpu, oracle, K):
    p1, gens = oracle.generators(K - 1)
    pts = [p1] + gens
    rows = [rand_scalars(b"cp%d" % K, b"r%d" % r, K) for r in range(33)]
    got = gpu.g1_msm_common_points(pts, rows)
    for row, (code, route, out) in zip(rows, got):
        assert code == 0 and route == 2 and out == oracle.g1_msm(pts, row)
    fused = gpu.g1_msm_common_points(pts, rows[:3], fused=True)
    assert [x[2] for x in fused] == [x[2] for x in got[:3]]


def test_common_points_scaled_rows(gpu, oracle):
    p1, gens = oracle.generators(9)
    pts = [p1] + gens
    rows = [rand_scalars(b"scaled", b"r%d" % r, 10) for r in range(4)]
    scales = rand_scalars(b"scaled", b"scale", 4)
    got = gpu.g1_msm_common_points(pts, rows, packed_scale=scales)
    for row, sc, (code, _, out) in zip(rows, scales, got):
        want = oracle.g1_msm(pts, [oracle.fr_mul(s, sc) for s in row])
        assert code == 0 and out == want


def test_common_points_arbitrary(gpu, oracle):
    pts = rand_points(oracle, b"arb", 7)
    rows = [rand_scalars(b"arb", b"r%d" % r, 7) for r in range(5)]
    got = gpu.g1_msm_common_points(pts, rows)
    for row, (code, route, out) in zip(rows, got):
        assert code == 0 and route == 4 and out == oracle.g1_msm(pts, row)


def test_common_points_plus_variable(gpu, oracle):
    p1, gens = oracle.generators(5)
    pts = [p1] + gens
    rows = [rand_scalars(b"cpv", b"r%d" % r, 6) for r in range(4)]
    vp = rand_points(oracle, b"cpv", 4)
    vs = rand_scalars(b"cpv", b"v", 4)
    got = gpu.g1_msm_common_points_plus_variable(pts, rows, vp, vs)
    for r, (code, out) in enumerate(got):
        assert code == 0 and out == oracle.g1_msm(pts + [vp[r]], rows[r] + [vs[r]])


def test_proof_verify_msm_pair(gpu, oracle):
    p1, gens = oracle.generators(11)
    pts = [p1] + gens
    rows = [rand_scalars(b"pair", b"r%d" % r, 12) for r in range(3)]
    pp = [rand_points(oracle, b"pp%d" % r, 3) for r in range(3)]
    ps = [rand_scalars(b"pair", b"s%d" % r, 4) for r in range(3)]
    got = gpu.proof_verify_msm_pair(pts, rows, pp, ps)
    for r, (code, t1, t2) in enumerate(got):
        assert code == 0
        assert t1 == oracle.g1_msm(pp[r], ps[r][:3])
        assert t2 == oracle.g1_msm(pts + [pp[r][2]], rows[r] + [ps[r][3]])


def test_dual_msm(gpu, oracle):
    pts = rand_points(oracle, b"dual", 9)
    lhs = rand_scalars(b"dual", b"l", 9)
    rhs = rand_scalars(b"dual", b"r", 9)
    code, a, b = gpu.g1_dual_msm_same_points(pts, lhs, rhs)
    assert code == 0 and a == oracle.g1_msm(pts, lhs) and b == oracle.g1_msm(pts, rhs)
    code, la, lb = gpu.g1_dual_msm_same_points(pts, lhs, rhs, lanes=3)
    assert code == 0
    for j in range(3):
        assert la[j] == oracle.g1_msm(pts[j::3], lhs[j::3])
        assert lb[j] == oracle.g1_msm(pts[j::3], rhs[j::3])


def test_g1_add(gpu, oracle):
    p = rand_points(oracle, b"add", 4)
    neg0 = bytes([p[0][0] ^ 0x20]) + p[0][1:]
    ident = bytes([0xC0]) + bytes(47)
    pairs = [(p[0], p[1]), (p[2], p[2]), (p[0], neg0), (ident, p[3]), (ident, ident)]
    got = gpu.g1_add_batch(pairs)
    for (a, b), (code, out) in zip(pairs, got):
        assert code == 0 and out == oracle.g1_add(a, b)


def test_decode_rejects_non_subgroup(gpu, oracle):
    # find x with x^3 + 4 square but the point outside G1: decompression must fail
    bad = []
    for i in range(64):
        x = int.from_bytes(drbg(b"nosub", b"x", i, 48), "big") % oracle.P_MOD
        enc = bytearray(x.to_bytes(48, "big"))
        enc[0] |= 0x80
        enc = bytes(enc)
        if oracle.g1_decompress(enc) is None:
            bad.append(enc)
        if len(bad) == 6:
            break
    one = (1).to_bytes(32, "big")
    got = gpu.g1_msm_batch([([b], [one]) for b in bad])
    assert all(code == gpu.ERR_INVALID_INPUT for code, _ in got)


def test_t2_prepare(gpu, oracle):
    p = rand_points(oracle, b"t2", 2)
    B, A = p
    s = rand_scalars(b"t2", b"s", 7)
    (code, d, abar, bbar, t1), = gpu.proof_gen_t2_prepare([(B, A, s)])
    negA = bytes([A[0] ^ 0x20]) + A[1:]
    assert code == 0
    assert d == oracle.g1_mul(B, s[0])
    assert abar == oracle.g1_mul(A, s[1])
    assert bbar == oracle.g1_msm([B, negA], [s[2], s[3]])
    assert t1 == oracle.g1_msm([A, B], [s[4], s[5]])


def test_pairing_eq(gpu, oracle):
    _, pk = keypair(oracle, b"pair")
    p1, _ = oracle.generators(1)
    k = scalar(b"pair", b"k", 0)
    a = oracle.g1_mul(p1, k)
    # e(k P1, PK) == e(P1, k PK) is not available without G2 mul; use e(a, PK) == e(a, PK)
    _, pk2 = keypair(oracle, b"pair", 1)
    reqs = [(a, pk, a, pk), (a, pk, a, pk2), (a, pk, p1, pk)]
    got = gpu.pairing_eq_batch(reqs)
    want = [oracle.pairing_eq(*r) == 0 for r in reqs]
    assert [v for _, v in got] == want == [True, False, False]


def test_pairing_eq_aggregate(gpu, oracle):
    _, pk = keypair(oracle, b"agg")
    _, pk2 = keypair(oracle, b"agg", 1)
    p = rand_points(oracle, b"agg", 3)
    c = rand_scalars(b"agg", b"c", 3)
    good = [(p[i], pk, p[i], pk, c[i]) for i in range(3)]
    assert gpu.pairing_eq_aggregate(good) == (0, True)
    bad = good[:2] + [(p[2], pk, p[2], pk2, c[2])]
    assert gpu.pairing_eq_aggregate(bad) == (0, False)


def test_g1_msm_batch_uneven_engine(gpu, oracle):
    """64 MSMs of uneven length take the persistent bucket-method engine."""
    import random
    rng = random.Random(11)
    seed = b"msm-uneven"
    p1, _ = oracle.generators(1)
    msms = []
    for i in range(64):
        K = rng.randint(2, 40)
        pts = [oracle.g1_mul(p1, scalar(seed, b"pt%d" % i, k)) for k in range(K)]
        scs = [scalar(seed, b"k%d" % i, k) for k in range(K)]
        if i == 5:
            pts[1] = bytes([0xC0]) + bytes(47)  # identity term
        if i == 9:
            scs[0] = bytes(32)                  # zero scalar
        msms.append((pts, scs))
    got = gpu.g1_msm_batch(msms)
    assert [(c, p) for c, p in got] == [(0, oracle.g1_msm(pts, scs)) for pts, scs in msms]


def test_msm_uneven_bench_self_check(gpu):
    r = gpu.msm_uneven_bench(n_msms=512, k_min=2, k_max=257, seed=9, tune=False, warmup=1, steps=1)
    assert r["checked"] == 64 and r["mismatch"] == 0 and r["ms"][0] > 0
