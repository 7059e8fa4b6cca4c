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


@pytest.mark.parametrize("coalesce_us,batch", [(2000, 128), (0, 4)])
def test_batcher_client_results_equal_alone(gpu, pool_and_alone, coalesce_us, batch):
    """The queue as the W3C batcher's replacement: per-operation batcher
    settings (window, batch size, capacity, pipelines under the shared slots),
    one request per enqueue with a reply callback or a receive, results equal
    to each request alone, and the snapshot counting every dispatch."""
    pool, alone = pool_and_alone
    rng = random.Random(11)
    order = list(range(len(pool)))
    rng.shuffle(order)
    with gpu.ServeQueue(max_inflight=4) as q:
        for op in (gpu.OP_SIGN, gpu.OP_VERIFY, gpu.OP_PROOF_GEN, gpu.OP_PROOF_VERIFY):
            q.configure(op, max_batch_items=batch, max_inflight=2, coalesce_us=coalesce_us, queue_capacity=64)
        replies = {}
        recs = []
        for i in order:
            op, req, sd = pool[i]
            recs.append((i, q.enqueue_request(op, req, seed=sd,
                                              callback=lambda reply, i=i: replies.__setitem__(i, reply))))
        for i, rec in recs:
            code, value, _ = rec.receive(60)
            op = pool[i][0]
            got = (code, rec.output()) if op in (gpu.OP_SIGN, gpu.OP_PROOF_GEN) else (code, bool(value))
            assert got == alone[i], (i, op)
            assert replies[i][0] == code
        total = q.snapshot(-1)
        assert total["dispatched_items"] == len(pool) and total["queued"] == 0
        for op in range(4):
            s = q.snapshot(op)
            n = sum(1 for o, _, _ in pool if o == op)
            assert s["dispatched_items"] == n
            assert sum(k * c for k, c in enumerate(s["batch_size_counts"])) == n
            assert s["max_observed_batch"] <= batch


def test_batcher_client_shake256_queues(gpu, pool_and_alone):
    """Queues 4..7 serve the same operations under BLS12-381-SHAKE-256: each
    reply equals the SHAKE-256 batch entry on the same request alone."""
    pool, _ = pool_and_alone
    sub = pool[:16]
    with gpu.ServeQueue(max_inflight=2) as q:
        for op in range(4):
            q.configure(gpu.serve_queue(op, gpu.SUITE_SHAKE256), max_batch_items=8, coalesce_us=500)
        recs = [q.enqueue_request(op, req, seed=sd, suite=gpu.SUITE_SHAKE256) for op, req, sd in sub]
        for (op, req, sd), rec in zip(sub, recs):
            code, value, _ = rec.receive(60)
            if op == gpu.OP_SIGN:
                assert (code, rec.output()) == tuple(gpu.sign_batch([req], suite=gpu.SUITE_SHAKE256)[0])
            elif op == gpu.OP_PROOF_GEN:
                want = gpu.proof_gen_batch([req], seeds=[sd], suite=gpu.SUITE_SHAKE256)[0]
                assert (code, rec.output()) == tuple(want)
            elif op == gpu.OP_VERIFY:
                assert (code, bool(value)) == tuple(gpu.verify_batch([req], suite=gpu.SUITE_SHAKE256)[0])
            else:
                assert (code, bool(value)) == tuple(gpu.proof_verify_batch([req], suite=gpu.SUITE_SHAKE256)[0])
        assert q.snapshot(-1)["dispatched_items"] == len(sub)
        assert sum(q.snapshot(op)["dispatched_items"] for op in range(4)) == 0
