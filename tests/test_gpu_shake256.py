"""GPU parity for the BLS12-381-SHAKE-256 ciphersuite (BBS_BLS12381G1_XOF:
SHAKE-256_SSWU_RO_, crates/cubbs-bbs-protocol/src/bbsplus/ciphersuites.rs:49-63)
through the *_batch_cs_v2 entry points: the CFRG fixture_data/bls12-381-shake-256
vectors (h2s, map-to-scalar, signatures, proofs byte for byte with the mocked
RNG) and random batches against the oracle's SHAKE-256 suite.  Bit-exact."""
import json

import pytest

from conftest import ROOT
from helpers import disclosed_subset, drbg, keypair, messages

h = bytes.fromhex
pytestmark = pytest.mark.gpu
SHAKE = 1
G = json.loads((ROOT / "tests" / "golden" / "cfrg_bls12381_shake256.json").read_text())


def test_expand_message_xof_and_h2s(gpu, oracle):
    dst = b"QUUX-V01-CS02-with-expander-SHAKE256"
    msgs = [drbg(b"xof", b"m", n, n) for n in (0, 1, 3, 64, 135, 136, 137, 300, 1000)]
    assert gpu.expand_xmd48_batch(msgs, dst, suite=SHAKE) == [oracle.expand_message_xof(m, dst, 48) for m in msgs]
    g = G["h2s"]
    assert gpu.hash_to_scalar_batch([h(g["message"])], h(g["dst"]), suite=SHAKE)[0].hex() == g["scalar"]
    m2s = G["MapMessageToScalarAsHash"]
    got = gpu.hash_to_scalar_batch([h(c["message"]) for c in m2s["cases"]], h(m2s["dst"]), suite=SHAKE)
    assert [x.hex() for x in got] == [c["scalar"] for c in m2s["cases"]]


def test_sign_fixtures(gpu):
    reqs, want = [], []
    for c in G["signature"]:
        if c["result"]["valid"]:
            reqs.append((h(c["signerKeyPair"]["secretKey"]), h(c["signerKeyPair"]["publicKey"]), h(c["header"]),
                         [h(m) for m in c["messages"]]))
            want.append(c["signature"])
    got = gpu.sign_batch(reqs, suite=SHAKE)
    assert [(code, sig.hex()) for code, sig in got] == [(0, w) for w in want]


def test_verify_fixtures(gpu):
    cases = G["signature"]
    reqs = [(h(c["signerKeyPair"]["publicKey"]), h(c["signature"]), h(c["header"]), [h(m) for m in c["messages"]])
            for c in cases]
    got = gpu.verify_batch(reqs, suite=SHAKE)
    assert all(code == 0 for code, _ in got)
    assert [v for _, v in got] == [c["result"]["valid"] for c in cases]


def test_proof_gen_fixtures(gpu, oracle):
    reqs, want = [], []
    for c in G["proof"]:
        if c["result"]["valid"]:
            reqs.append((h(c["signerPublicKey"]), h(c["signature"]), h(c["header"]), h(c["presentationHeader"]),
                         [h(m) for m in c["messages"]], c["disclosedIndexes"]))
            want.append(c["proof"])
    got = gpu.proof_gen_batch(reqs, seeds=[oracle.SEED_MOCKED_SCALAR] * len(reqs), suite=SHAKE)
    assert [(code, p.hex()) for code, p in got] == [(0, w) for w in want]


def test_proof_verify_fixtures(gpu):
    reqs, want = [], []
    for c in G["proof"]:
        msgs = [h(m) for m in c["messages"]]
        di = c["disclosedIndexes"]
        reqs.append((h(c["signerPublicKey"]), h(c["proof"]), h(c["header"]), h(c["presentationHeader"]),
                     [msgs[i] for i in di if i < len(msgs)], di, len(msgs)))
        want.append(c["result"]["valid"])
    got = gpu.proof_verify_batch(reqs, suite=SHAKE)
    assert [v for _, v in got] == want


@pytest.mark.parametrize("L,R", [(1, 0), (10, 5), (100, 50), (200, 20)])
def test_roundtrip_random_against_oracle(gpu, oracle, L, R):
    """Sign, Verify, ProofGen (seeded) and ProofVerify of random batches equal the
    oracle's SHAKE-256 suite byte for byte; L = 200 at 20 disclosed draws 185
    blinding scalars from one expand_message_xof call."""
    seed = b"shake-%d-%d" % (L, R)
    reqs = []
    for i in range(4):
        sk, pk = keypair(oracle, seed, i % 2)
        reqs.append((sk, pk, drbg(seed, b"hdr", i, 64), messages(seed, i, L, 48)))
    sigs = gpu.sign_batch(reqs, suite=SHAKE)
    for (sk, pk, hdr, msgs), (code, sig) in zip(reqs, sigs):
        assert code == 0 and sig == oracle.sign(sk, pk, hdr, msgs, suite=SHAKE)[0]
    vreqs = [(pk, sig, hdr, msgs) for (sk, pk, hdr, msgs), (_, sig) in zip(reqs, sigs)]
    vreqs += [(pk, sig, hdr + b"!", msgs) for (sk, pk, hdr, msgs), (_, sig) in zip(reqs, sigs)]
    assert [v for _, v in gpu.verify_batch(vreqs, suite=SHAKE)] == [True] * 4 + [False] * 4
    preqs, seeds = [], []
    for i, ((sk, pk, hdr, msgs), (_, sig)) in enumerate(zip(reqs, sigs)):
        preqs.append((pk, sig, hdr, drbg(seed, b"ph", i, 32), msgs, disclosed_subset(seed, i, L, R)))
        seeds.append(drbg(seed, b"seed", i, 32))
    proofs = gpu.proof_gen_batch(preqs, seeds=seeds, suite=SHAKE)
    pv = []
    for (pk, sig, hdr, ph, msgs, di), sd, (code, proof) in zip(preqs, seeds, proofs):
        assert code == 0
        assert proof == oracle.proof_gen(pk, sig, hdr, ph, msgs, di, seed=sd, suite=SHAKE)
        pv.append((pk, proof, hdr, ph, [msgs[j] for j in di], di, L))
        pv.append((pk, proof, hdr, ph + b"?", [msgs[j] for j in di], di, L))
    assert [v for _, v in gpu.proof_verify_batch(pv, suite=SHAKE)] == [True, False] * 4


def test_aggregated_group_and_suite_separation(gpu, oracle):
    """130 SHAKE-256 proofs under one key (an aggregated key group, with one
    pairing-only failure) verify as the oracle says; the same proofs under the
    SHA-256 entry point, and SHA-256 signatures under the SHAKE-256 one, fail."""
    seed = b"shake-agg"
    sk, pk = keypair(oracle, seed)
    items = []
    for i in range(130):
        msgs = messages(seed, i, 6, 32)
        sig = oracle.sign(sk, pk, b"h", msgs, suite=SHAKE)[0]
        if i == 17:
            sig = oracle.sign(sk, pk, b"h", messages(seed + b"-o", i, 6, 32), suite=SHAKE)[0][:48] + sig[48:]
        di = disclosed_subset(seed, i, 6, 3)
        proof = oracle.proof_gen(pk, sig, b"h", b"p", msgs, di, seed=drbg(seed, b"s", i, 32), suite=SHAKE)
        items.append((pk, proof, b"h", b"p", [msgs[j] for j in di], di, 6))
    want = [oracle.proof_verify(*it[:6], suite=SHAKE) == 0 for it in items]
    assert want.count(False) == 1 and want[17] is False
    assert [v for _, v in gpu.proof_verify_batch(items, suite=SHAKE)] == want
    assert not any(v for _, v in gpu.proof_verify_batch(items[:20]))
    msgs = messages(seed, 999, 5, 32)
    sha_sig = oracle.sign(sk, pk, b"h", msgs)[0]
    assert gpu.verify_batch([(pk, sha_sig, b"h", msgs)], suite=SHAKE)[0][1] is False
    assert gpu.verify_batch([(pk, sha_sig, b"h", msgs)])[0][1] is True


def test_unknown_suite_is_rejected(gpu):
    import ctypes
    lib = gpu.lib()
    res = (gpu.Result * 1)()
    assert lib.cubbs_bbs_gpu_verify_batch_cs_v2(2, 7, None, 0, ctypes.cast(res, ctypes.c_void_p)) == \
        gpu.ERR_INVALID_INPUT
    assert lib.cubbs_bbs_gpu_verify_batch_cs_v2(2, 1, None, 0, ctypes.cast(res, ctypes.c_void_p)) == gpu.SUCCESS
