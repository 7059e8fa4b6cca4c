"""GPU parity on the benchmark configurations and the edge cases around them,
through the C ABI against the oracle (bit-exact):

* the uneven variable-base MSM engine (16384-MSM workload's K ~ U{2..257})
  on MSMs from every size class, under the autotuned settings and under every
  forced (chunk, window) setting the engine accepts;
* the fixed-base MSM (4096 x 12-term workload) at every table width 4..20;
* ProofVerify at the headline shape (1024 proofs, L = 100, 50 disclosed) over
  several keys, with about 2 % invalid items of several kinds;
* proofs whose Abar, Bbar or D is the identity encoding, which the reference
  parses (G1Affine::from_compressed accepts 0xc0 00..00:
  crates/cubbs-bbs-protocol/src/utils/util.rs:53-62, bbsplus/proof.rs:189-195),
  alone and inside aggregated key groups."""
import concurrent.futures as cf
import os
import random

import pytest

from helpers import R_MOD, disclosed_subset, drbg, keypair, messages, scalar

pytestmark = pytest.mark.gpu
IDENT = bytes([0xC0]) + bytes(47)
THREADS = max(2, os.cpu_count() or 2)


def pmap(fn, args):
    """The oracle's calls release the GIL: run them on all host cores."""
    with cf.ThreadPoolExecutor(max_workers=THREADS) as ex:
        return list(ex.map(lambda a: fn(*a), args))


# ----------------------------------------------------------------------------- uneven MSM engine
def _uneven_msms(oracle, seed, n=64):
    """n MSMs whose term counts cover every size class of the engine (K <= 8,
    <= 32, <= 96, larger, up to 257), over a pool of 300 random points; a few
    identity points and zero scalars."""
    rng = random.Random(seed)
    p1, _ = oracle.generators(1)
    pool = pmap(lambda i: oracle.g1_mul(p1, scalar(b"c4-pool", b"pt", i)), [(i,) for i in range(300)])
    edges = [2, 8, 9, 32, 33, 96, 97, 257]
    msms = []
    for i in range(n):
        K = edges[i] if i < len(edges) else rng.randint(2, 257)
        off = rng.randrange(300)
        pts = [pool[(off + 7 * k) % 300] for k in range(K)]
        scs = [scalar(b"c4-%d" % seed, b"k%d" % i, k) for k in range(K)]
        if i % 11 == 3:
            pts[K // 2] = IDENT
        if i % 13 == 5:
            scs[0] = bytes(32)
        msms.append((pts, scs))
    want = pmap(oracle.g1_msm, msms)
    return msms, want


def test_uneven_msm_engine_every_setting(gpu, oracle):
    """The engine (taken by g1_msm_batch_v2 for 32+ MSMs of 8+ terms each) under
    the autotuned settings, in thread mode under every window 4..7 with chunk
    lengths from one term per lane to whole MSMs, in warp mode (one warp per
    MSM, shared buckets) under every window 4..12, and with the modes mixed per
    size class: every output equals the oracle's."""
    msms, want = _uneven_msms(oracle, 21)
    saved = gpu.msm_tuning()
    try:
        r = gpu.msm_uneven_bench(n_msms=2048, k_min=2, k_max=257, seed=5, tune=True, warmup=0, steps=1)
        assert r["mismatch"] == 0
        tuned = gpu.msm_tuning()
        assert tuned == (r["chunk"], r["window"], r["mode"])
        got = gpu.g1_msm_batch(msms)
        assert got == [(0, w) for w in want], "autotuned %s" % (tuned,)
        for c in (4, 5, 6, 7):
            for t in (1, 3, 16, 64, 256):
                gpu.msm_tuning([t] * 4, [c] * 4, [0] * 4)
                got = gpu.g1_msm_batch(msms)
                assert got == [(0, w) for w in want], "thread mode, chunk %d window %d" % (t, c)
        for c in range(4, 13):
            gpu.msm_tuning([8] * 4, [c] * 4, [1] * 4)
            got = gpu.g1_msm_batch(msms)
            assert got == [(0, w) for w in want], "warp mode, window %d" % c
        # mixed settings per size class
        gpu.msm_tuning([2, 8, 24, 40], [7, 4, 6, 5], [0, 0, 0, 0])
        assert gpu.g1_msm_batch(msms) == [(0, w) for w in want]
        gpu.msm_tuning([2, 8, 24, 40], [5, 9, 6, 11], [0, 1, 0, 1])
        assert gpu.g1_msm_batch(msms) == [(0, w) for w in want]
    finally:
        gpu.msm_tuning(*saved)


def test_msm_tuning_rejects_out_of_range(gpu):
    with pytest.raises(ValueError):
        gpu.msm_tuning([8, 8, 8, 8], [3, 4, 4, 4])
    with pytest.raises(ValueError):
        gpu.msm_tuning([0, 8, 8, 8], [4, 4, 4, 4])
    with pytest.raises(ValueError):  # thread mode stops at window 7
        gpu.msm_tuning([8, 8, 8, 8], [8, 4, 4, 4], [0, 0, 0, 0])
    with pytest.raises(ValueError):  # warp mode stops at window 12
        gpu.msm_tuning([8, 8, 8, 8], [13, 4, 4, 4], [1, 0, 0, 0])


# ----------------------------------------------------------------------------- fixed-base MSM widths
def test_fixed_msm_every_table_width(gpu, oracle):
    """The 12-term fixed-base MSM over [P1, Q1, H1..H10] at every table width
    4..20 (the autotuner's sweep with one width selects it): each width's
    output equals the oracle's, and the autotuner's own check finds no width
    that disagrees."""
    p1, gens = oracle.generators(11)
    pts = [p1] + gens
    rows = [[scalar(b"c2-widths", b"r%d" % r, k) for k in range(12)] for r in range(40)]
    rows[3][5] = bytes(32)
    rows[7] = [(R_MOD - 1).to_bytes(32, "big")] * 12
    want = pmap(oracle.g1_msm, [(pts, row) for row in rows])
    flat = b"".join(b"".join(row) for row in rows)
    before = gpu.table_window()
    seen = set()
    try:
        for w in range(4, 21):
            ms, best, bad = gpu.fixed_msm_autotune(flat, len(rows), 12, w, w, steps=1, with_mismatches=True)
            assert bad == 0 and best == w and ms[0] > 0
            # a table too large for the budget is narrowed (only possible at the widest widths)
            got_w = gpu.table_window()
            assert got_w == w or (w > 16 and 16 <= got_w < w)
            seen.add(got_w)
            got = gpu.g1_msm_common_points(pts, rows)
            assert [(c, route, out) for c, route, out in got] == [(0, 2, x) for x in want], "width %d" % w
        assert set(range(4, 17)) <= seen
        ms, best, bad = gpu.fixed_msm_autotune(flat, len(rows), 12, 4, 20, steps=1, with_mismatches=True)
        assert bad == 0 and 4 <= best <= 20 and all(m > 0 for m in ms)
    finally:
        restore = before if before else 16
        gpu.fixed_msm_autotune(flat, len(rows), 12, restore, restore, steps=1)


# ----------------------------------------------------------------------------- ProofVerify, headline shape
def test_proof_verify_headline_shape_multi_key(gpu, oracle):
    """1024 proofs at L = 100 (64-byte messages), 50 disclosed, over 8 keys
    (aggregated key groups of about 128), with 20 invalid items: proofs from a
    signature on other messages (pass the challenge, fail only the pairing),
    changed presentation headers, tampered responses, the wrong public key and
    a non-canonical response scalar.  ProofGen runs on the device (a sample is
    compared byte for byte with the oracle); every verdict equals the oracle's."""
    seed = b"headline-1024"
    L, R, N, KEYS = 100, 50, 1024, 8
    keys = [keypair(oracle, seed, k) for k in range(KEYS)]
    hdrs = [drbg(seed, b"hdr", i, 64) for i in range(N)]
    msgs = [messages(seed, i, L, 64) for i in range(N)]
    fake = set(range(37, N, 170))  # 6 items signed over other messages
    sign_args = [(keys[i % KEYS][0], keys[i % KEYS][1], hdrs[i],
                  messages(seed + b"-other", i, L, 64) if i in fake else msgs[i]) for i in range(N)]
    sigs = [r[0] for r in pmap(oracle.sign, sign_args)]
    for i in fake:  # A over other messages with the e of the right ones: passes the challenge only
        sigs[i] = sigs[i][:48] + oracle.sign(keys[i % KEYS][0], keys[i % KEYS][1], hdrs[i], msgs[i])[0][48:]
    dis = [disclosed_subset(seed, i, L, R) for i in range(N)]
    phs = [drbg(seed, b"ph", i, 64) for i in range(N)]
    pseeds = [drbg(seed, b"pseed", i, 32) for i in range(N)]
    reqs = [(keys[i % KEYS][1], sigs[i], hdrs[i], phs[i], msgs[i], dis[i]) for i in range(N)]
    gen = gpu.proof_gen_batch(reqs, seeds=pseeds)
    assert all(c == 0 for c, _ in gen)
    proofs = [p for _, p in gen]
    sample = list(range(0, N, 64)) + sorted(fake)
    want_pg = pmap(lambda i: oracle.proof_gen(*reqs[i], seed=pseeds[i]), [(i,) for i in sample])
    assert [proofs[i] for i in sample] == want_pg
    items = [(keys[i % KEYS][1], proofs[i], hdrs[i], phs[i], [msgs[i][j] for j in dis[i]], dis[i], L)
             for i in range(N)]
    for i in range(101, N, 170):  # 6 changed presentation headers
        items[i] = items[i][:3] + (items[i][3] + b"!",) + items[i][4:]
    for i in range(5, N, 256):  # 4 tampered responses (an m^ changed)
        p = items[i][1]
        items[i] = items[i][:1] + (p[:300] + bytes([p[300] ^ 0x10]) + p[301:],) + items[i][2:]
    for i in (222, 777):  # verified under another key
        items[i] = (keys[(i + 1) % KEYS][1],) + items[i][1:]
    for i in (400, 900):  # a response that is not a canonical scalar
        p = items[i][1]
        items[i] = items[i][:1] + (p[:240] + R_MOD.to_bytes(32, "big") + p[272:],) + items[i][2:]
    want = [v == 0 for v in pmap(oracle.proof_verify, [it[:6] for it in items])]
    assert want.count(False) == 20
    got = gpu.proof_verify_batch(items)
    assert all(c == 0 for c, _ in got)
    assert [v for _, v in got] == want


# ----------------------------------------------------------------------------- identity points in proofs
def _forged_identity_proof(oracle, pk, hdr, ph, msgs, di, tag):
    """A proof with Abar = Bbar = identity that passes the challenge check
    without any signature: T1 = D r1^ does not depend on c, and with
    D = delta * Bv (Bv = P1 + Q1 domain + sum_{i in R} H_i m_i, which the
    verifier recomputes) T2 = t Bv + sum_j H_j m^_j once r3^ = (t - c) / delta.
    The pairing terms are both the identity, so the reference accepts it."""
    L = len(msgs)
    p1, gens = oracle.generators(L + 1)
    dom = int.from_bytes(oracle.calculate_domain(pk, hdr, L), "big")
    m = [int.from_bytes(oracle.hash_to_scalar(x, oracle.MAP_DST), "big") for x in msgs]
    und = [j for j in range(L) if j not in di]
    rnd = [int.from_bytes(scalar(b"forge", tag, k), "big") for k in range(4 + len(und))]
    delta, t, r1h, eh = rnd[:4]
    mh = rnd[4:]
    be = lambda v: (v % R_MOD).to_bytes(32, "big")
    Bv = oracle.g1_msm([p1, gens[0]] + [gens[1 + i] for i in di], [be(1), be(dom)] + [be(m[i]) for i in di])
    D = oracle.g1_mul(Bv, be(delta))
    T1 = oracle.g1_mul(D, be(r1h))
    T2 = oracle.g1_msm([Bv] + [gens[1 + j] for j in und], [be(t)] + [be(x) for x in mh])
    c_in = len(di).to_bytes(8, "big")
    for i in di:
        c_in += i.to_bytes(8, "big") + be(m[i])
    c_in += IDENT + IDENT + D + T1 + T2 + be(dom) + len(ph).to_bytes(8, "big") + ph
    c = int.from_bytes(oracle.hash_to_scalar(c_in, oracle.H2S_DST), "big")
    r3h = (t - c) * pow(delta, -1, R_MOD)
    return IDENT + IDENT + D + be(eh) + be(r1h) + be(r3h) + b"".join(be(x) for x in mh) + be(c)


def test_proof_verify_identity_points(gpu, oracle):
    """Identity Abar, Bbar, D (and pairs of them) substituted into honest proofs,
    plus forged proofs with Abar = Bbar = identity that pass the challenge: the
    verdicts equal the oracle's (which follows the reference, where the forged
    ones verify), inside an aggregated key group of valid proofs, inside a
    group's fallback, and alone."""
    seed = b"identity-pv"
    sk, pk = keypair(oracle, seed)
    L = 8
    base = []
    for i in range(140):
        ms = messages(seed, i, L, 32)
        sig = oracle.sign(sk, pk, b"h", ms)[0]
        di = disclosed_subset(seed, i, L, 3)
        proof = oracle.proof_gen(pk, sig, b"h", b"p", ms, di, seed=drbg(seed, b"s", i, 32))
        base.append((pk, proof, b"h", b"p", [ms[j] for j in di], di, L))
    cases = []
    for k, (pk_, pr, hd, ph, dm, di, L_) in enumerate(base[:7]):
        parts = [pr[0:48], pr[48:96], pr[96:144]]
        for slot in ([0], [1], [2], [0, 1], [1, 2], [0, 1, 2], [])[k:k + 1]:
            q = list(parts)
            for s in slot:
                q[s] = IDENT
            cases.append((pk_, b"".join(q) + pr[144:], hd, ph, dm, di, L_))
    for k in range(3):
        ms = messages(seed + b"-forge", k, L, 32)
        di = disclosed_subset(seed + b"-forge", k, L, 2 + k)
        proof = _forged_identity_proof(oracle, pk, b"h", b"p", ms, di, b"%d" % k)
        cases.append((pk, proof, b"h", b"p", [ms[j] for j in di], di, L))
    want_cases = [oracle.proof_verify(*c[:6]) == 0 for c in cases]
    assert want_cases[-3:] == [True] * 3, "the forged identity proofs verify under the oracle"
    assert want_cases[:7] == [False] * 6 + [True]
    # alone (batches too small to group)
    assert [v for _, v in gpu.proof_verify_batch(cases)] == want_cases
    for c, w in zip(cases, want_cases):
        assert gpu.proof_verify_batch([c])[0][1] == w
    # inside a key group of valid proofs (the group check passes: identity terms add nothing)
    batch = base[7:] + cases
    want = [True] * len(base[7:]) + want_cases
    assert [v for _, v in gpu.proof_verify_batch(batch)] == want
    # inside a group that fails (a pairing-only failure forces the per-item fallback)
    fake_sig = oracle.sign(sk, pk, b"h", messages(seed + b"-x", 0, L, 32))[0][:48]
    ms = messages(seed, 500, L, 32)
    sig = fake_sig + oracle.sign(sk, pk, b"h", ms)[0][48:]
    bad = oracle.proof_gen(pk, sig, b"h", b"p", ms, [0], seed=b"f" * 32)
    batch2 = batch + [(pk, bad, b"h", b"p", [ms[0]], [0], L)]
    want2 = want + [oracle.proof_verify(pk, bad, b"h", b"p", [ms[0]], [0]) == 0]
    assert want2[-1] is False
    assert [v for _, v in gpu.proof_verify_batch(batch2)] == want2


def test_msms_and_pairings_in_one_launch(gpu, oracle):
    """An uneven batch of MSMs (sizes across every class, thread and warp units)
    and pairing checks (true, false, identity and undecodable inputs) through
    one persistent launch: every result equals the oracle's and the separate
    entry points'; the same call again replays the engine's captured graph."""
    msms, want = _uneven_msms(oracle, 33, n=40)
    _, pk = keypair(oracle, b"mixed")
    _, pk2 = keypair(oracle, b"mixed", 1)
    p1, _ = oracle.generators(1)
    a = oracle.g1_mul(p1, scalar(b"mixed", b"a", 0))
    bad_g1 = bytes([a[0] ^ 0x01]) + a[1:]
    pairs = [(a, pk, a, pk), (a, pk, a, pk2), (a, pk, p1, pk), (IDENT, pk, IDENT, pk2), (bad_g1, pk, a, pk)]
    want_p = [(0, True), (0, False), (0, False), (0, True), (1, False)]
    assert [oracle.pairing_eq(*r) == 0 for r in pairs[:4]] == [True, False, False, True]
    saved = gpu.msm_tuning()
    try:
        for mode in ([0, 0, 0, 0], [1, 1, 1, 1], [0, 1, 0, 1]):
            gpu.msm_tuning([8, 16, 32, 48], [5, 6, 6, 7], mode)
            for _ in range(2):
                got_m, got_p = gpu.g1_msm_pairing_batch(msms, pairs)
                assert got_m == [(0, w) for w in want], mode
                assert [(c, v if c == 0 else False) for c, v in got_p] == want_p
        assert gpu.g1_msm_pairing_batch([], pairs)[1] == gpu.pairing_eq_batch(pairs)
        assert gpu.g1_msm_pairing_batch(msms[:3], [])[0] == gpu.g1_msm_batch(msms[:3])
    finally:
        gpu.msm_tuning(*saved)
