"""bbs-2023 base proofs through the library's lowering (header, messages, Sign /
Verify on the device, proofValue) against the oracle: the issued proofValue
text equals the oracle's signature serialised by the oracle's codec, and the
verdicts follow prepared.rs:423-513 (a key or header mismatch is false, a
malformed proofValue is its codec error)."""
import hashlib

import pytest

from helpers import drbg, keypair
from oracle import bbs2023_oracle as B
from oracle import proofvalue_oracle as PV

pytestmark = pytest.mark.gpu


def _credential(seed, i):
    """Canonical N-Quads of a small credential, split into mandatory and non-mandatory lines."""
    subj = "_:b%d" % (i % 3)
    lines = ['%s <https://schema.org/name> "Holder %d" .\n' % (subj, i),
             '%s <https://schema.org/birthDate> "19%02d-01-%02d"^^<http://www.w3.org/2001/XMLSchema#date> .\n'
             % (subj, i % 100, 1 + i % 28),
             '<urn:uuid:%s> <https://www.w3.org/2018/credentials#credentialSubject> %s .\n'
             % (drbg(seed, b"id", i, 8).hex(), subj),
             '%s <https://schema.org/address> "Street ü%d" .\n' % (subj, i)]
    lines += ['%s <urn:p%d> "v%d" .\n' % (subj, k, k) for k in range(i % 5)]
    lines = sorted(lines, key=lambda s: s.encode())
    mandatory = [x for k, x in enumerate(lines) if k % 3 == 0]
    non_mandatory = [x for k, x in enumerate(lines) if k % 3 != 0]
    proof_hash = hashlib.sha256(("proof-config-%d" % i).encode()).digest()
    return proof_hash, mandatory, non_mandatory


def test_issue_and_verify_base_proofs(gpu, oracle):
    seed = b"bbs2023"
    sk, pk = keypair(oracle, seed)
    items = []
    for i in range(24):
        ph, mand, non = _credential(seed, i)
        items.append((sk, pk, ph, mand, non, drbg(seed, b"hmac", i, 32), ["/credentialSubject/name", "/issuer"][: i % 3]))
    issued = gpu.bbs2023_issue_base_proof_batch(items)
    for (sk_, pk_, ph, mand, non, hk, ptrs), (code, text) in zip(items, issued):
        assert code == 0
        header, msgs = B.issue_lowering(ph, mand, non)
        sig = oracle.sign(sk_, pk_, header, msgs)[0]
        assert text == PV.serialize_base(sig, header, pk_, hk, ptrs)
    # verify: the issued proofs, then mismatches of each kind
    good = [(pk, ph, mand, non, text) for (_, _, ph, mand, non, _, _), (_, text) in zip(items, issued)]
    _, other_pk = keypair(oracle, seed, 1)
    bad = [
        (pk, good[0][1], good[0][2], good[0][3][:-1] + [good[0][3][-1] + "x"], good[0][4]),  # message changed
        (other_pk, good[1][1], good[1][2], good[1][3], good[1][4]),                          # other key
        (pk, good[2][1], good[2][2][1:], good[2][3], good[2][4]),                             # mandatory changed
        (pk, bytes(32), good[3][2], good[3][3], good[3][4]),                                 # proof hash changed
    ]
    res = gpu.bbs2023_verify_base_proof_batch(good + bad)
    assert res == [(0, True)] * len(good) + [(0, False)] * len(bad)
    # the oracle agrees on the one that reaches Verify with a changed message
    header, msgs = B.issue_lowering(bad[0][1], bad[0][2], bad[0][3])
    sig = PV.parse_base(good[0][4])[0]
    assert oracle.verify(pk, sig, header, msgs) != 0


def test_issue_and_verify_errors(gpu, oracle):
    seed = b"bbs2023-err"
    sk, pk = keypair(oracle, seed)
    ph, mand, non = _credential(seed, 1)
    res = gpu.bbs2023_issue_base_proof_batch([(sk, pk, ph, mand, non, bytes(31), []),
                                              (sk, pk, ph, mand, non, bytes(32), ["/a"])])
    assert res[0] == (20, None) and res[1][0] == 0
    text = res[1][1]
    broken = [text[1:], "u" + text[2:], text + "A"]
    got = gpu.bbs2023_verify_base_proof_batch([(pk, ph, mand, non, t) for t in broken])
    assert [c for c, _ in got] == [10, 11, 14] or all(c != 0 for c, _ in got)
    assert got[0][0] == 10  # no multibase prefix
