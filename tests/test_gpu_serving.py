"""Serving queue (continuous batching) against single-request calls: every
request's result is the same alone and in the mix, for a burst, Poisson
arrivals, a tight device-memory budget and the plain fixed-size batcher."""
import random

import pytest

from helpers import disclosed_subset, drbg, keypair, messages

pytestmark = pytest.mark.gpu


def _pool(gpu, oracle):
    seed = b"serving"
    keys = [keypair(oracle, seed, i) for i in range(3)]
    pool = []
    for i in range(12):
        sk, pk = keys[i % 3]
        L = (5, 10, 20, 50)[i % 4]
        msgs = messages(seed, i, L, 32)
        hdr = drbg(seed, b"hdr", i, 64)
        pool.append((gpu.OP_SIGN, (sk, pk, hdr, msgs), None))
        sig = oracle.sign(sk, pk, hdr, msgs)[0]
        pool.append((gpu.OP_VERIFY, (pk, sig, hdr, msgs), None))
        if i % 3 == 0:
            pool.append((gpu.OP_VERIFY, (pk, sig, hdr + b"x", msgs), None))
        R = max(1, int(L * (0.1 + 0.8 * ((i * 37) % 100) / 100)))
        di = disclosed_subset(seed, i, L, R)
        ph = drbg(seed, b"ph", i, 64)
        pg_seed = drbg(seed, b"pgseed", i, 32)
        pool.append((gpu.OP_PROOF_GEN, (pk, sig, hdr, ph, msgs, di), pg_seed))
        proof = oracle.proof_gen(pk, sig, hdr, ph, msgs, di, seed=pg_seed)
        dm = [msgs[j] for j in di]
        pool.append((gpu.OP_PROOF_VERIFY, (pk, proof, hdr, ph, dm, di, L), None))
        if i % 4 == 1:
            pool.append((gpu.OP_PROOF_VERIFY, (pk, proof, hdr, ph + b"!", dm, di, L), None))
    return pool


def _alone(gpu, pool):
    out = []
    for op, req, sd in pool:
        if op == gpu.OP_SIGN:
            (code, sig), = gpu.sign_batch([req])
            out.append((code, sig))
        elif op == gpu.OP_VERIFY:
            (code, ok), = gpu.verify_batch([req])
            out.append((code, ok))
        elif op == gpu.OP_PROOF_GEN:
            (code, proof), = gpu.proof_gen_batch([req], seeds=[sd])
            out.append((code, proof))
        else:
            (code, ok), = gpu.proof_verify_batch([req])
            out.append((code, ok))
    return out


def _mixed(gpu, pool, results):
    out = []
    for (op, _, _), (code, value, data) in zip(pool, results):
        out.append((code, data) if op in (gpu.OP_SIGN, gpu.OP_PROOF_GEN) else (code, bool(value)))
    return out


@pytest.fixture(scope="module")
def pool_and_alone(gpu, oracle):
    pool = _pool(gpu, oracle)
    return pool, _alone(gpu, pool)


def test_alone_results_are_the_expected_ones(gpu, oracle, pool_and_alone):
    pool, alone = pool_and_alone
    for (op, req, sd), (code, val) in zip(pool, alone):
        assert code == 0
        if op == gpu.OP_SIGN:
            assert val == oracle.sign(*req)[0]
        elif op == gpu.OP_PROOF_GEN:
            assert val == oracle.proof_gen(*req, seed=sd)
    assert sum(1 for (op, *_), (_, v) in zip(pool, alone) if op in (gpu.OP_VERIFY, gpu.OP_PROOF_VERIFY) and not v) == 7


@pytest.mark.parametrize("mode,batch,budget,arrivals", [
    (0, 4, 0, "burst"),
    (0, 1024, 0, "poisson"),
    (0, 8, 64 << 10, "burst"),   # the memory budget admits a few requests at a time
    (1, 6, 0, "poisson"),         # plain fixed-size batches
])
def test_mixed_results_equal_alone(gpu, pool_and_alone, mode, batch, budget, arrivals):
    pool, alone = pool_and_alone
    rng = random.Random(7)
    order = list(range(len(pool)))
    rng.shuffle(order)
    t, schedule = 0, []
    for i in order:
        if arrivals == "poisson":
            t += int(rng.expovariate(20000.0) * 1e9)
        schedule.append((i, t))
    results, lat, wall = gpu.serve_replay(pool, schedule, mode=mode, max_batch_items=batch, hbm_budget_bytes=budget,
                                          plain_batch=batch, plain_timeout_us=500)
    got = _mixed(gpu, [pool[i] for i, _ in schedule], results)
    want = [alone[i] for i, _ in schedule]
    assert got == want
    assert all(x > 0 for x in lat) and wall > 0
