"""The CPU oracle's SHAKE-256 ciphersuite (BBS_BLS12381G1_XOF:SHAKE-256_SSWU_RO_,
crates/cubbs-bbs-protocol/src/bbsplus/ciphersuites.rs:49-63) against the
reference's CFRG fixture_data/bls12-381-shake-256 (h2s, MapMessageToScalarAsHash,
generators, mockedRng, keypair, signature001-010, proof001-015), and its SHAKE-256
against Python's hashlib (CPU only)."""
import hashlib
import json

import pytest

from conftest import ROOT
from helpers import disclosed_subset, keypair, messages

h = bytes.fromhex
SHAKE = 1
G = json.loads((ROOT / "tests" / "golden" / "cfrg_bls12381_shake256.json").read_text())


@pytest.mark.parametrize("n", [0, 1, 135, 136, 137, 271, 272, 1000])
def test_shake256_matches_hashlib(oracle, n):
    msg = bytes((7 * i + n) & 0xFF for i in range(n))
    for out in (32, 48, 136, 137, 300):
        assert oracle.shake256(msg, out) == hashlib.shake_256(msg).digest(out)


def test_expand_message_xof_definition(oracle):
    """RFC 9380 5.3.2: SHAKE256(msg || I2OSP(n, 2) || DST || I2OSP(len(DST), 1), n)."""
    dst = b"QUUX-V01-CS02-with-expander-SHAKE256"
    for msg in (b"", b"abc", b"a" * 512):
        for n in (32, 48, 128, 0x80 + 1):
            want = hashlib.shake_256(msg + n.to_bytes(2, "big") + dst + bytes([len(dst)])).digest(n)
            assert oracle.expand_message_xof(msg, dst, n) == want


def test_hash_to_scalar_fixture(oracle):
    g = G["h2s"]
    assert oracle.hash_to_scalar(h(g["message"]), h(g["dst"]), suite=SHAKE).hex() == g["scalar"]


def test_map_message_to_scalar_fixture(oracle):
    g = G["MapMessageToScalarAsHash"]
    for case in g["cases"]:
        assert oracle.hash_to_scalar(h(case["message"]), h(g["dst"]), suite=SHAKE).hex() == case["scalar"]


def test_generators_fixture(oracle):
    p1, gens = oracle.generators(11, suite=SHAKE)
    g = G["generators"]
    assert p1.hex() == g["P1"]
    assert gens[0].hex() == g["Q1"]
    assert [x.hex() for x in gens[1:]] == g["MsgGenerators"]


def test_mocked_rng_fixture(oracle):
    g = G["mockedRng"]
    got = oracle.seeded_random_scalars(h(g["seed"]), h(g["dst"]), g["count"], suite=SHAKE)
    assert [x.hex() for x in got] == g["mockedScalars"]


def test_keypair_fixture(oracle):
    g = G["keypair"]
    sk = oracle.keygen(h(g["keyMaterial"]), h(g["keyInfo"]), h(g["keyDst"]), suite=SHAKE)
    assert sk.hex() == g["keyPair"]["secretKey"]
    assert oracle.sk_to_pk(sk).hex() == g["keyPair"]["publicKey"]


@pytest.mark.parametrize("idx", range(10))
def test_signature_fixtures(oracle, idx):
    c = G["signature"][idx]
    pk = h(c["signerKeyPair"]["publicKey"])
    sk = h(c["signerKeyPair"]["secretKey"])
    msgs = [h(m) for m in c["messages"]]
    hdr = h(c["header"])
    rc = oracle.verify(pk, h(c["signature"]), hdr, msgs, suite=SHAKE)
    assert (rc == 0) == c["result"]["valid"]
    if c["result"]["valid"]:
        sig, b, dom = oracle.sign(sk, pk, hdr, msgs, suite=SHAKE)
        assert sig.hex() == c["signature"]
        assert b.hex() == c["trace"]["B"]
        assert dom.hex() == c["trace"]["domain"]


@pytest.mark.parametrize("idx", range(15))
def test_proof_fixtures(oracle, idx):
    c = G["proof"][idx]
    pk = h(c["signerPublicKey"])
    msgs = [h(m) for m in c["messages"]]
    di = c["disclosedIndexes"]
    hdr, ph = h(c["header"]), h(c["presentationHeader"])
    if c["result"]["valid"]:
        proof = oracle.proof_gen(pk, h(c["signature"]), hdr, ph, msgs, di, suite=SHAKE)
        assert proof.hex() == c["proof"]
    dmsgs = [msgs[i] for i in di if i < len(msgs)]
    rc = oracle.proof_verify(pk, h(c["proof"]), hdr, ph, dmsgs, di, suite=SHAKE)
    assert (rc == 0) == c["result"]["valid"]


def test_suites_differ_and_do_not_leak(oracle):
    """The suite is per call: a SHAKE-256 call leaves the thread on SHA-256, and a
    SHA-256 signature does not verify under SHAKE-256."""
    seed = b"oracle-suites"
    sk, pk = keypair(oracle, seed)
    msgs = messages(seed, 0, 12, 32)
    sig_sha = oracle.sign(sk, pk, b"h", msgs)[0]
    sig_shake = oracle.sign(sk, pk, b"h", msgs, suite=SHAKE)[0]
    assert sig_sha != sig_shake
    assert oracle.verify(pk, sig_sha, b"h", msgs) == 0
    assert oracle.verify(pk, sig_shake, b"h", msgs, suite=SHAKE) == 0
    assert oracle.verify(pk, sig_sha, b"h", msgs, suite=SHAKE) == 2
    di = disclosed_subset(seed, 0, 12, 5)
    proof = oracle.proof_gen(pk, sig_shake, b"h", b"p", msgs, di, seed=b"z" * 32, suite=SHAKE)
    assert oracle.proof_verify(pk, proof, b"h", b"p", [msgs[i] for i in di], di, suite=SHAKE) == 0
    assert oracle.proof_verify(pk, proof, b"h", b"p", [msgs[i] for i in di], di) == 2


def test_unchunked_random_scalars_past_170(oracle):
    """expand_message_xof takes up to 65535 bytes: 200 scalars come from one call,
    so the first 170 are not a chunk of their own (unlike expand_message_xmd)."""
    a = oracle.seeded_random_scalars(b"x" * 32, b"dst", 200, suite=SHAKE)
    b = oracle.seeded_random_scalars(b"x" * 32, b"dst", 170, suite=SHAKE)
    assert len(set(a)) == 200
    # one squeeze: the 170-scalar stream is not a prefix of the 200 (the length is hashed in)
    assert a[:170] != b
