"""GPU parity: the sm_103a library through its C ABI against the CPU oracle and
the golden vectors.  Integer/byte work, so every comparison is bit-exact."""
import pytest

from helpers import disclosed_subset, drbg, keypair, messages, scalar

h = bytes.fromhex
pytestmark = pytest.mark.gpu


# ----------------------------------------------------------------------------- hashing
def test_sha256_kats(gpu, golden):
    kat = golden["sha256_kat"]
    got = gpu.sha256_batch([m.encode() for m in kat["messages"]])
    assert [g.hex() for g in got] == kat["digests"]


def test_sha256_lengths(gpu, oracle):
    msgs = [drbg(b"sha", b"len", n, n) for n in (0, 1, 55, 56, 63, 64, 65, 119, 120, 1000)]
    assert gpu.sha256_batch(msgs) == [oracle.sha256(m) for m in msgs]


def test_expand_xmd48(gpu, oracle):
    dst = b"QUUX-V01-CS02-with-expander-SHA256-128"
    msgs = [drbg(b"xmd", b"m", n, n) for n in (0, 3, 64, 200)]
    assert gpu.expand_xmd48_batch(msgs, dst) == [oracle.expand_message_xmd(m, dst, 48) for m in msgs]


def test_hash_to_scalar_fixture(gpu, golden):
    g = golden["h2s"]
    assert gpu.hash_to_scalar_batch([h(g["message"])], h(g["dst"]))[0].hex() == g["scalar"]


def test_messages_to_scalar_fixture(gpu, golden):
    g = golden["MapMessageToScalarAsHash"]
    got = gpu.messages_to_scalar([h(c["message"]) for c in g["cases"]], h(g["dst"]))
    assert [x.hex() for x in got] == [c["scalar"] for c in g["cases"]]


# ----------------------------------------------------------------------------- Sign / Verify
def test_sign_fixtures(gpu, golden):
    reqs, want = [], []
    for c in golden["signature"]:
        if c["result"]["valid"]:
            reqs.append((h(c["signerKeyPair"]["secretKey"]), h(c["signerKeyPair"]["publicKey"]), h(c["header"]),
                         [h(m) for m in c["messages"]]))
            want.append(c["signature"])
    got = gpu.sign_batch(reqs)
    assert [(code, sig.hex()) for code, sig in got] == [(0, w) for w in want]


def test_verify_fixtures(gpu, golden):
    cases = golden["signature"]
    reqs = [(h(c["signerKeyPair"]["publicKey"]), h(c["signature"]), h(c["header"]), [h(m) for m in c["messages"]])
            for c in cases]
    got = gpu.verify_batch(reqs)
    assert [v for _, v in got] == [c["result"]["valid"] for c in cases]
    assert all(code == 0 for code, _ in got)


@pytest.mark.parametrize("L", [1, 10, 100])
def test_sign_verify_random(gpu, oracle, L):
    seed = b"sign-verify-%d" % L
    reqs, vreqs = [], []
    for i in range(8):
        sk, pk = keypair(oracle, seed, i % 3)
        msgs = messages(seed, i, L, 32)
        hdr = drbg(seed, b"hdr", i, 64)
        reqs.append((sk, pk, hdr, msgs))
    got = gpu.sign_batch(reqs)
    for (sk, pk, hdr, msgs), (code, sig) in zip(reqs, got):
        assert code == 0
        assert sig == oracle.sign(sk, pk, hdr, msgs)[0]
        vreqs.append((pk, sig, hdr, msgs))
        vreqs.append((pk, sig, hdr, msgs[::-1] if L > 1 else [b"x"]))
    ver = gpu.verify_batch(vreqs)
    assert [v for _, v in ver] == [True, False] * len(reqs)


def test_verify_rejects_malformed(gpu, oracle):
    seed = b"verify-bad"
    sk, pk = keypair(oracle, seed)
    msgs = messages(seed, 0, 5, 32)
    sig = oracle.sign(sk, pk, b"", msgs)[0]
    bad_e = sig[:48] + (0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001).to_bytes(32, "big")
    not_on_curve = bytes([sig[0] ^ 0x01]) + sig[1:]
    ident = bytes([0xC0]) + bytes(47) + sig[48:]
    got = gpu.verify_batch([(pk, bad_e, b"", msgs), (pk, sig[:79], b"", msgs), (pk, ident, b"", msgs),
                            (pk, sig, b"", msgs)])
    assert [v for _, v in got] == [False, False, False, True]
    # an off-curve / non-subgroup A never verifies
    assert gpu.verify_batch([(pk, not_on_curve, b"", msgs)])[0][1] is False
    # an undecodable public key is an item error
    bad_pk = bytes([pk[0] ^ 0x01]) + pk[1:]
    code, _ = gpu.verify_batch([(bad_pk, sig, b"", msgs)])[0]
    assert code == gpu.ERR_INVALID_INPUT


# ----------------------------------------------------------------------------- ProofGen / ProofVerify
def test_proof_gen_fixtures(gpu, golden, oracle):
    reqs, want = [], []
    for c in golden["proof"]:
        if c["result"]["valid"]:
            reqs.append((h(c["signerPublicKey"]), h(c["signature"]), h(c["header"]), h(c["presentationHeader"]),
                         [h(m) for m in c["messages"]], c["disclosedIndexes"]))
            want.append(c["proof"])
    got = gpu.proof_gen_batch(reqs, seeds=[oracle.SEED_MOCKED_SCALAR] * len(reqs))
    assert [(code, p.hex()) for code, p in got] == [(0, w) for w in want]


def test_proof_verify_fixtures(gpu, golden):
    reqs, want = [], []
    for c in golden["proof"]:
        msgs = [h(m) for m in c["messages"]]
        di = c["disclosedIndexes"]
        reqs.append((h(c["signerPublicKey"]), h(c["proof"]), h(c["header"]), h(c["presentationHeader"]),
                     [msgs[i] for i in di if i < len(msgs)], di, len(msgs)))
        want.append(c["result"]["valid"])
    got = gpu.proof_verify_batch(reqs)
    assert [v for _, v in got] == want


@pytest.mark.parametrize("L,R", [(10, 5), (100, 50), (100, 0), (100, 100), (30, 29)])
def test_proof_roundtrip_random(gpu, oracle, L, R):
    seed = b"proof-%d-%d" % (L, R)
    sk, pk = keypair(oracle, seed)
    reqs, seeds = [], []
    for i in range(6):
        msgs = messages(seed, i, L, 64)
        hdr = drbg(seed, b"hdr", i, 64)
        sig = oracle.sign(sk, pk, hdr, msgs)[0]
        di = disclosed_subset(seed, i, L, R)
        ph = drbg(seed, b"ph", i, 64)
        reqs.append((pk, sig, hdr, ph, msgs, di))
        seeds.append(drbg(seed, b"seed", i, 32))
    got = gpu.proof_gen_batch(reqs, seeds=seeds)
    vreqs = []
    for (pk_, sig, hdr, ph, msgs, di), sd, (code, proof) in zip(reqs, seeds, got):
        assert code == 0
        assert proof == oracle.proof_gen(pk_, sig, hdr, ph, msgs, di, seed=sd)
        dm = [msgs[j] for j in di]
        vreqs.append((pk_, proof, hdr, ph, dm, di, L))
        vreqs.append((pk_, proof, hdr, ph + b"!", dm, di, L))
    ver = gpu.proof_verify_batch(vreqs)
    assert [v for _, v in ver] == [True, False] * len(reqs)


def test_proof_gen_chunked_random_scalars(gpu, oracle):
    """L = 200 with 10 disclosed: 5 + U = 195 blinding scalars exceed one
    expand_message call (255 x 32 bytes), so they are drawn in chunks; bytes equal
    the oracle's, and the proofs verify (generators beyond the first 128)."""
    seed = b"proof-chunked"
    sk, pk = keypair(oracle, seed)
    reqs, seeds = [], []
    for i in range(3):
        msgs = messages(seed, i, 200, 32)
        sig = oracle.sign(sk, pk, b"h", msgs)[0]
        di = disclosed_subset(seed, i, 200, 10)
        reqs.append((pk, sig, b"h", b"p", msgs, di))
        seeds.append(drbg(seed, b"seed", i, 32))
    got = gpu.proof_gen_batch(reqs, seeds=seeds)
    for (pk_, sig, hdr, ph, msgs, di), sd, (code, proof) in zip(reqs, seeds, got):
        assert code == 0 and proof == oracle.proof_gen(pk_, sig, hdr, ph, msgs, di, seed=sd)
    ver = gpu.proof_verify_batch([(pk_, proof, hdr, ph, [msgs[j] for j in di], di, 200)
                                  for (pk_, sig, hdr, ph, msgs, di), (_, proof) in zip(reqs, got)])
    assert all(c == 0 and v for c, v in ver)


def test_empty_batches(gpu):
    """A batch of zero items succeeds without touching the device."""
    import ctypes
    lib = gpu.lib()
    res = (gpu.Result * 1)()
    for name in ("sign", "verify", "proof_gen", "proof_verify"):
        fn = getattr(lib, "cubbs_bbs_gpu_%s_batch_v2" % name)
        fn.restype = ctypes.c_int32
        fn.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        assert fn(2, None, 0, ctypes.cast(res, ctypes.c_void_p)) == 0, name


def test_proof_gen_os_randomness_verifies(gpu, oracle):
    seed = b"proof-os"
    sk, pk = keypair(oracle, seed)
    msgs = messages(seed, 0, 12, 32)
    sig = oracle.sign(sk, pk, b"h", msgs)[0]
    di = [0, 3, 7]
    (c1, p1), (c2, p2) = gpu.proof_gen_batch([(pk, sig, b"h", b"p", msgs, di)] * 2)
    assert c1 == 0 and c2 == 0 and p1 != p2
    for p in (p1, p2):
        assert oracle.proof_verify(pk, p, b"h", b"p", [msgs[j] for j in di], di) == 0


def test_proof_verify_tampered(gpu, oracle):
    seed = b"proof-tamper"
    sk, pk = keypair(oracle, seed)
    msgs = messages(seed, 0, 20, 32)
    sig = oracle.sign(sk, pk, b"h", msgs)[0]
    di = [1, 2, 5, 19]
    proof = oracle.proof_gen(pk, sig, b"h", b"p", msgs, di, seed=b"t" * 32)
    dm = [msgs[j] for j in di]
    flips = [proof[:200] + bytes([proof[200] ^ 1]) + proof[201:],  # r1^ changed
             proof[:-1] + bytes([proof[-1] ^ 1]),                    # challenge changed
             bytes([proof[0] ^ 0x20]) + proof[1:],                   # Abar negated
             proof[:-32],                                            # truncated
             proof + b"\x00" * 5]                                    # trailing bytes ignored as the reference does
    reqs = [(pk, f, b"h", b"p", dm, di, 20) for f in flips] + [(pk, proof, b"h", b"p", dm[::-1], di, 20)]
    got = [v for _, v in gpu.proof_verify_batch(reqs)]
    want = [oracle.proof_verify(pk, f, b"h", b"p", dm, di) == 0 for f in flips] + [False]
    assert got == want
    assert want[-2] is True and not any(want[:4])


def _on_curve_outside_g1(oracle, tag):
    """Compressed encoding of a point of E(Fp): y^2 = x^3 + 4 whose x comes from a
    hash; such a point lies in G1 with probability 1/h, h ~ 2^126."""
    P = oracle.P_MOD
    ctr = 0
    while True:
        x = int.from_bytes(drbg(b"non-g1", tag, ctr, 64), "big") % P
        ctr += 1
        rhs = (x * x * x + 4) % P
        y = pow(rhs, (P + 1) // 4, P)
        if y * y % P == rhs:
            b = bytearray(x.to_bytes(48, "big"))
            b[0] |= 0x80 | (0x20 if y > P - y else 0)
            return bytes(b)


def test_proof_verify_rejects_points_outside_g1(gpu, oracle):
    """Abar, Bbar or D on the curve but outside G1: rejected like the oracle does."""
    seed = b"proof-non-g1"
    sk, pk = keypair(oracle, seed)
    msgs = messages(seed, 0, 16, 32)
    sig = oracle.sign(sk, pk, b"h", msgs)[0]
    di = [0, 4, 9]
    proof = oracle.proof_gen(pk, sig, b"h", b"p", msgs, di, seed=b"g" * 32)
    dm = [msgs[j] for j in di]
    bad = [proof[:48 * k] + _on_curve_outside_g1(oracle, b"%d" % k) + proof[48 * (k + 1):] for k in range(3)]
    reqs = [(pk, f, b"h", b"p", dm, di, 16) for f in bad + [proof]]
    got = [v for _, v in gpu.proof_verify_batch(reqs)]
    want = [oracle.proof_verify(pk, f, b"h", b"p", dm, di) == 0 for f in bad + [proof]]
    assert want == [False, False, False, True]
    assert got == want


def test_split_subgroup_check(gpu, golden, oracle):
    """The unchecked decode plus the separate subgroup kernel used by ProofVerify:
    G1 points pass, curve points outside G1 are flagged, undecodable ones fail decode."""
    g = golden["generators"]
    in_g1 = [h(x) for x in [g["P1"], g["Q1"]] + g["MsgGenerators"]]
    sk, pk = keypair(oracle, b"subgroup")
    in_g1 += [oracle.sign(sk, pk, b"", messages(b"subgroup", i, 3, 32))[0][:48] for i in range(4)]
    outside = [_on_curve_outside_g1(oracle, b"s%d" % i) for i in range(8)]
    undecodable = [bytes([in_g1[0][0] ^ 0x01]) + in_g1[0][1:]]
    got = gpu.g1_subgroup_for_test(in_g1 + outside + undecodable)
    assert got[:len(in_g1)] == [(0, 0)] * len(in_g1)
    assert got[len(in_g1):len(in_g1) + len(outside)] == [(0, 1)] * len(outside)
    assert got[-1][0] == 2 and got[-1][1] == 0


def _pv_items(oracle, seed, count, L, fake=()):
    """`count` ProofVerify items under one key; items in `fake` are proofs made
    from the signature of other messages, which pass the challenge check and
    fail only the pairing check."""
    sk, pk = keypair(oracle, seed)
    items = []
    for i in range(count):
        msgs = messages(seed, i, L, 32)
        sig = oracle.sign(sk, pk, b"h", msgs)[0]
        if i in fake:
            sig = oracle.sign(sk, pk, b"h", messages(seed + b"-other", i, L, 32))[0][:48] + sig[48:]
        di = disclosed_subset(seed, i, L, L // 2)
        proof = oracle.proof_gen(pk, sig, b"h", b"p", msgs, di, seed=drbg(seed, b"s", i, 32))
        items.append((pk, proof, b"h", b"p", [msgs[j] for j in di], di, L))
    return items


def test_proof_verify_aggregated_groups(gpu, oracle):
    """Batches of 128 or more check each key's proofs (16 or more) as one group;
    a group that fails is checked item by item.  Every verdict equals the
    oracle's and the verdict of the same item in a batch too small to group.
    266 items also take the multi-threaded packing of the call."""
    big = _pv_items(oracle, b"agg-a", 236, 6, fake={5, 77, 130, 201})
    small = _pv_items(oracle, b"agg-b", 10, 6, fake={3})
    clean = _pv_items(oracle, b"agg-c", 20, 6)
    items = big + small + clean
    items[40] = items[40][:3] + (b"p!",) + items[40][4:]   # challenge mismatch
    items[150] = items[150][:1] + (items[150][1][:200],) + items[150][2:]  # too short: rejected by shape
    want = [oracle.proof_verify(pk, pr, hd, ph, dm, di) == 0 for pk, pr, hd, ph, dm, di, _ in items]
    assert want.count(False) == 7
    got = [v for _, v in gpu.proof_verify_batch(items)]
    assert got == want
    alone = []
    for k in range(0, len(items), 50):
        alone += [v for _, v in gpu.proof_verify_batch(items[k:k + 50])]
    assert alone == want
    # all valid: every group check passes
    ok_items = [it for it, w in zip(items, want) if w]
    assert all(v for _, v in gpu.proof_verify_batch(ok_items))


def test_proof_verify_bucket_groups(gpu, oracle):
    """A key group of 256 items or more takes the bucket MSM for its group sums
    (smaller groups one ladder per point): with pairing-only failures and a
    challenge mismatch inside the 300-item group every verdict equals the
    oracle's, and the group of the valid items passes its check."""
    items = _pv_items(oracle, b"bucket-a", 300, 6, fake={11, 150, 299}) + \
        _pv_items(oracle, b"bucket-b", 20, 6, fake={4})
    items[60] = items[60][:3] + (b"p!",) + items[60][4:]   # challenge mismatch
    want = [oracle.proof_verify(pk, pr, hd, ph, dm, di) == 0 for pk, pr, hd, ph, dm, di, _ in items]
    assert want.count(False) == 5
    got = [v for _, v in gpu.proof_verify_batch(items)]
    assert got == want
    ok_items = [it for it, w in zip(items, want) if w]
    assert all(v for _, v in gpu.proof_verify_batch(ok_items))


def test_verify_bucket_groups(gpu, oracle):
    """Verify with a 280-item key group (bucket MSM for the group sums): a
    signature over other messages and one with a changed e inside the group;
    every verdict equals the oracle's."""
    seed = b"verify-bucket"
    sk, pk = keypair(oracle, seed, 0)
    items = []
    for i in range(280):
        msgs = messages(seed, i, 4, 32)
        items.append((pk, oracle.sign(sk, pk, b"hdr", msgs)[0], b"hdr", msgs))
    items[9] = (pk, items[9][1], b"hdr", messages(seed + b"-o", 9, 4, 32))
    e = (int.from_bytes(items[200][1][48:], "big") + 1).to_bytes(32, "big")
    items[200] = (pk, items[200][1][:48] + e, b"hdr", items[200][3])
    want = [oracle.verify(*it) == 0 for it in items]
    assert want.count(False) == 2
    assert [v for _, v in gpu.verify_batch(items)] == want
    ok_items = [it for it, w in zip(items, want) if w]
    assert all(v for _, v in gpu.verify_batch(ok_items))


def test_sign_e_resident(gpu, oracle):
    import ctypes
    seed = b"sign-e"
    sk, pk = keypair(oracle, seed)
    msgs = messages(seed, 0, 6, 32)
    dom = scalar(seed, b"dom", 0)
    k = gpu._Keep()
    item = gpu.SignEFromResidentScalarsItem()
    item.secret_key = k.bytes(sk)
    item.domain = k.bytes(dom)
    item.messages = k.slices(msgs)
    item.message_scalar_offset = 0
    item.message_count = len(msgs)
    mo, mbuf = k.out(32 * len(msgs))
    eo, ebuf = k.out(32)
    item.message_scalars_out = mo
    item.scalar_out = eo
    res = (gpu.Result * 1)()
    rc = gpu.lib().cubbs_bbs_gpu_sign_e_from_resident_scalars_batch_v2(
        2, ctypes.cast(ctypes.pointer(item), ctypes.c_void_p), 1, k.bytes(gpu.MAP_DST), k.bytes(gpu.H2S_DST),
        ctypes.cast(res, ctypes.c_void_p))
    assert rc == 0 and res[0].code == 0
    scal = [oracle.hash_to_scalar(m, gpu.MAP_DST) for m in msgs]
    assert mbuf.raw[:32 * len(msgs)] == b"".join(scal)
    assert ebuf.raw[:32] == oracle.hash_to_scalar(sk + b"".join(scal) + dom, gpu.H2S_DST)


def test_sign_parts(gpu, oracle, golden):
    c = golden["signature"][0]
    sk, pk = h(c["signerKeyPair"]["secretKey"]), h(c["signerKeyPair"]["publicKey"])
    msgs, hdr = [h(m) for m in c["messages"]], h(c["header"])
    (code, sig), = gpu.sign_batch([(sk, pk, hdr, msgs)])
    want = h(c["signature"])
    assert (code, sig[48:].hex()) == (0, want[48:].hex()), "e differs"
    assert sig[:48].hex() == want[:48].hex(), "A differs"


def test_verify_aggregated_groups(gpu, oracle):
    """Verify batches of 128 or more check each key's signatures (16 or more) as
    one random-coefficient group and fall back to per-item checks when a group
    fails.  Groups with failing items (signatures over other messages, a changed
    header, a changed e, A outside G1, the identity A) and a passing group: every
    verdict equals the oracle's and the verdict of the same item in a batch too
    small to group."""
    seed = b"verify-agg"
    items = []
    for key in range(3):
        sk, pk = keypair(oracle, seed, key)
        for i in range(60 if key < 2 else 20):
            msgs = messages(seed, 100 * key + i, 8, 32)
            sig = oracle.sign(sk, pk, b"hdr", msgs)[0]
            items.append((pk, sig, b"hdr", msgs))
    pk0 = items[0][0]
    bad_msgs = messages(seed + b"-o", 0, 8, 32)
    items[3] = (pk0, items[3][1], b"hdr", bad_msgs)                       # other messages
    items[17] = (pk0, items[17][1], b"hdx", items[17][3])                 # changed header
    e = (int.from_bytes(items[29][1][48:], "big") + 1).to_bytes(32, "big")
    items[29] = (pk0, items[29][1][:48] + e, b"hdr", items[29][3])        # changed e
    items[41] = (pk0, _on_curve_outside_g1(oracle, b"vagg") + items[41][1][48:], b"hdr", items[41][3])
    items[77] = (items[77][0], bytes([0xC0]) + bytes(47) + items[77][1][48:], b"hdr", items[77][3])
    items[130] = (items[0][0], items[130][1], b"hdr", items[130][3])      # verified under another key
    want = [oracle.verify(*it) == 0 for it in items]
    assert want.count(False) == 6 and len(items) == 140
    got = gpu.verify_batch(items)
    assert [v for _, v in got] == want
    alone = []
    for k in range(0, len(items), 50):
        alone += [v for _, v in gpu.verify_batch(items[k:k + 50])]
    assert alone == want
    ok_items = [it for it, w in zip(items, want) if w]
    assert all(v for _, v in gpu.verify_batch(ok_items))
