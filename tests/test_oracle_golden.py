"""The CPU oracle against the reference's golden vectors (CPU only).

Pins: CFRG fixture_data/bls12-381-sha-256 (h2s, MapMessageToScalarAsHash,
generators, mockedRng, keypair, signature001-010, proof001-015) and the native
smoke KATs (native/cuda/tests/sha256_smoke.cpp, prepare_b_smoke.cpp).
"""
import pytest

from helpers import disclosed_subset, keypair, messages

h = bytes.fromhex


def test_sha256_kats(oracle, golden):
    kat = golden["sha256_kat"]
    for m, d in zip(kat["messages"], kat["digests"]):
        assert oracle.sha256(m.encode()).hex() == d


def test_hash_to_scalar_fixture(oracle, golden):
    g = golden["h2s"]
    assert oracle.hash_to_scalar(h(g["message"]), h(g["dst"])).hex() == g["scalar"]


def test_map_message_to_scalar_fixture(oracle, golden):
    g = golden["MapMessageToScalarAsHash"]
    for case in g["cases"]:
        assert oracle.hash_to_scalar(h(case["message"]), h(g["dst"])).hex() == case["scalar"]


def test_generators_fixture(oracle, golden):
    p1, gens = oracle.generators(11)
    g = golden["generators"]
    assert p1.hex() == g["P1"]
    assert gens[0].hex() == g["Q1"]
    assert [x.hex() for x in gens[1:]] == g["MsgGenerators"]


def test_mocked_rng_fixture(oracle, golden):
    g = golden["mockedRng"]
    got = oracle.seeded_random_scalars(h(g["seed"]), h(g["dst"]), g["count"])
    assert [x.hex() for x in got] == g["mockedScalars"]


def test_keypair_fixture(oracle, golden):
    g = golden["keypair"]
    sk = oracle.keygen(h(g["keyMaterial"]), h(g["keyInfo"]), h(g["keyDst"]))
    assert sk.hex() == g["keyPair"]["secretKey"]
    assert oracle.sk_to_pk(sk).hex() == g["keyPair"]["publicKey"]


@pytest.mark.parametrize("idx", range(10))
def test_signature_fixtures(oracle, golden, idx):
    c = golden["signature"][idx]
    pk = h(c["signerKeyPair"]["publicKey"])
    sk = h(c["signerKeyPair"]["secretKey"])
    msgs = [h(m) for m in c["messages"]]
    hdr = h(c["header"])
    rc = oracle.verify(pk, h(c["signature"]), hdr, msgs)
    assert (rc == 0) == c["result"]["valid"]
    if c["result"]["valid"]:
        sig, b, dom = oracle.sign(sk, pk, hdr, msgs)
        assert sig.hex() == c["signature"]
        assert b.hex() == c["trace"]["B"]
        assert dom.hex() == c["trace"]["domain"]


@pytest.mark.parametrize("idx", range(15))
def test_proof_fixtures(oracle, golden, idx):
    c = golden["proof"][idx]
    pk = h(c["signerPublicKey"])
    msgs = [h(m) for m in c["messages"]]
    di = c["disclosedIndexes"]
    hdr, ph = h(c["header"]), h(c["presentationHeader"])
    if c["result"]["valid"]:
        proof = oracle.proof_gen(pk, h(c["signature"]), hdr, ph, msgs, di)
        assert proof.hex() == c["proof"]
    dmsgs = [msgs[i] for i in di if i < len(msgs)]
    rc = oracle.proof_verify(pk, h(c["proof"]), hdr, ph, dmsgs, di)
    assert (rc == 0) == c["result"]["valid"]


def test_prepare_b_msm_kat(oracle, golden):
    k = golden["prepare_b_kat"]
    got = oracle.g1_msm([h(p) for p in k["msm_points"]], [h(s) for s in k["msm_scalars"]])
    assert got.hex() == k["expected_b"]
    # the points are [P1, Q1, H1..H4] and the second scalar is calculate_domain(PK, header, L=4)
    p1, gens = oracle.generators(5)
    assert [p1.hex()] + [g.hex() for g in gens] == k["msm_points"]
    assert oracle.calculate_domain(h(k["public_key"]), h(k["header"]), 4).hex() == k["msm_scalars"][1]
    assert k["msm_scalars"][2:] == k["message_scalars"]


def test_roundtrip_large_L(oracle):
    seed = b"oracle-roundtrip"
    sk, pk = keypair(oracle, seed)
    msgs = messages(seed, 0, 40, 64)
    sig, _, _ = oracle.sign(sk, pk, b"hdr", msgs)
    assert oracle.verify(pk, sig, b"hdr", msgs) == 0
    assert oracle.verify(pk, sig, b"hdr", msgs[::-1]) == 2
    di = disclosed_subset(seed, 0, 40, 20)
    proof = oracle.proof_gen(pk, sig, b"hdr", b"ph", msgs, di, seed=b"s" * 32)
    assert len(proof) == 272 + 32 * 20
    assert oracle.proof_verify(pk, proof, b"hdr", b"ph", [msgs[i] for i in di], di) == 0
    assert oracle.proof_verify(pk, proof, b"hdr", b"ph2", [msgs[i] for i in di], di) == 2


def test_chunked_random_scalars(oracle):
    # past 170 scalars the expansion is chunked; the first chunk keeps its own seed suffix
    a = oracle.seeded_random_scalars(b"x" * 32, b"dst", 171)
    assert len(a) == 171 and len(set(a)) == 171
    b = oracle.seeded_random_scalars(b"x" * 32, b"dst", 170)
    assert a[:170] != b  # chunked derivation is a different (documented) stream
