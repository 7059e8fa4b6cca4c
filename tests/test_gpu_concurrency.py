"""Concurrent ABI calls from several host threads (the Rust engine calls the
library from many threads): every result equals the same call made alone."""
import concurrent.futures as cf

import pytest

from helpers import disclosed_subset, drbg, keypair, messages, scalar

pytestmark = pytest.mark.gpu


def _workload(oracle):
    seed = b"concurrency"
    sk, pk = keypair(oracle, seed)
    sign_reqs = [(sk, pk, drbg(seed, b"hdr", i, 64), messages(seed, i, 10, 32)) for i in range(6)]
    sigs = [oracle.sign(*r)[0] for r in sign_reqs]
    verify_reqs = [(pk, s, r[2], r[3]) for s, r in zip(sigs, sign_reqs)]
    verify_reqs.append((pk, sigs[0], sign_reqs[1][2], sign_reqs[1][3]))  # wrong signature
    L = 20
    pg_reqs, seeds = [], []
    for i in range(4):
        msgs = messages(seed, 100 + i, L, 64)
        hdr = drbg(seed, b"pghdr", i, 64)
        sig = oracle.sign(sk, pk, hdr, msgs)[0]
        di = disclosed_subset(seed, i, L, 8)
        pg_reqs.append((pk, sig, hdr, drbg(seed, b"ph", i, 64), msgs, di))
        seeds.append(drbg(seed, b"seed", i, 32))
    proofs = [oracle.proof_gen(*r, seed=s) for r, s in zip(pg_reqs, seeds)]
    pv_reqs = [(r[0], p, r[2], r[3], [r[4][j] for j in r[5]], r[5], L) for r, p in zip(pg_reqs, proofs)]
    p1, _ = oracle.generators(1)
    msm = [([oracle.g1_mul(p1, scalar(seed, b"pt", 10 * i + k)) for k in range(5)],
            [scalar(seed, b"k", 10 * i + k) for k in range(5)]) for i in range(3)]
    return sign_reqs, verify_reqs, pg_reqs, seeds, pv_reqs, msm


def test_concurrent_calls_match_sequential(gpu, oracle):
    sign_reqs, verify_reqs, pg_reqs, seeds, pv_reqs, msm = _workload(oracle)
    calls = {
        "sign": lambda: gpu.sign_batch(sign_reqs),
        "verify": lambda: gpu.verify_batch(verify_reqs),
        "proof_gen": lambda: gpu.proof_gen_batch(pg_reqs, seeds=seeds),
        "proof_verify": lambda: gpu.proof_verify_batch(pv_reqs),
        "msm": lambda: gpu.g1_msm_batch(msm),
    }
    alone = {k: f() for k, f in calls.items()}
    assert [v for _, v in alone["verify"]] == [True] * 6 + [False]
    assert all(v for _, v in alone["proof_verify"])
    jobs = [k for k in calls for _ in range(4)]
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        futs = [(k, ex.submit(calls[k])) for k in jobs]
        for k, f in futs:
            assert f.result() == alone[k], k
