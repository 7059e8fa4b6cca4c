#!/usr/bin/env python3
"""BBS ProofVerify / ProofGen throughput at L=100 on GB300 (one JSON line).

Workload: BBS ProofGen + ProofVerify, BLS12-381-SHA-256, L = 100 messages of
64 random bytes, a seeded 50-message disclosed subset per proof, 1024 proofs
per batch (one step = one pass of the device pipeline over that batch).
Inputs are synthetic and seeded (SHA-256 counter DRBG); signatures and proofs
are produced by this library before timing.  Headline metric: ProofVerify
ops/s; ProofGen, Sign and Verify ops/s are reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

value       : device-resident pipeline throughput (inputs in HBM, CUDA events on
              the library stream, L2 flushed between steps)
e2e         : the same metric through the C ABI with host buffers (packing,
              H2D and D2H inside the timed region)
roofline    : the dominant stage vs the measured integer multiply-add peak
cpu_baseline: the CPU oracle (a port of the reference's Rust CPU path) on all
              host cores, on a bounded sample of the same workload
--impl reference: the same metric for the reference's CPU implementation of
              the path (the C++ oracle port; the Rust crates cannot be built
              here), run on rank 0 only.
"""
import argparse
import concurrent.futures as cf
import hashlib
import importlib.util
import json
import os
import pathlib
import statistics
import subprocess
import sys
import time

ROOT = pathlib.Path(__file__).resolve().parent
R_MOD = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001

# CFRG draft keypair fixture (keypair.json): one signer for the whole batch.
SK = bytes.fromhex("60e55110f76883a13d030b2f6bd11883422d5abde717569fc0731f51237169fc")
PK = bytes.fromhex("a820f230f6ae38503b86c70dc50b61c58a77e45c39ab25c0652bbaa8fa136f2851bd4781c9dcde39fc9d1d52c9e60268"
                   "061e7d7632171d91aa8d460acee0e96f1e7c4cfb12d3ff9ab5d5dc91c277db75c845d649ef3c4f63aebc364cd55ded0c")

# Frozen per-op work model in 381-bit Montgomery products (M); 1 M = 600 IMAD.
IMAD_PER_M = 600
MODEL_M = {
    "proof_verify": {"g1_decode": 3 * 1750, "fixed_msm": 102 * 260, "var_mul": 6700 + 2224, "challenge": 12,
                     "pairing": 16470, "pairing_kernel": 16470, "total": 57180},
    "proof_gen": {"g1_decode": 1750, "fixed_msm": 102 * 260 + 50 * 260, "var_mul": 12896 + 2224, "finish": 30,
                  "total": 56450},
}


# DRAM bytes per launch of a stage's kernel at this workload, from one ncu capture
# of the 1024-proof, L = 100 step (dram__bytes_read.sum + dram__bytes_write.sum):
# k_var_mul_pair moved 0.638 + 0.004 MB for its 4096 terms (points, scalars, jobs);
# k_fixed_msm<32> moved 170.4 + 3.5 MB with the table narrowed to window 14 (19
# windows per term, so that the capture fits); table reads scale with the windows,
# so the window-20 launch (13 windows) moves about 173.9 MB x 13 / 19 = 119 MB.
TRAFFIC_BYTES = {"fixed_msm": 173.9e6 * 13 / 19, "var_mul": 0.6415e6}


def drbg(seed: bytes, label: bytes, i: int, n: int) -> bytes:
    out, ctr = b"", 0
    while len(out) < n:
        out += hashlib.sha256(seed + label + i.to_bytes(8, "big") + ctr.to_bytes(4, "big")).digest()
        ctr += 1
    return out[:n]


def load_package():
    pkg = ROOT / "cubbs-cred_gb300"
    spec = importlib.util.spec_from_file_location("cubbs_gb300", pkg / "__init__.py",
                                                  submodule_search_locations=[str(pkg)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["cubbs_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def make_requests(n, L, R, msg_len, seed):
    """Per proof: messages, header, presentation header, sorted disclosed subset."""
    reqs = []
    for i in range(n):
        msgs = [drbg(seed, b"msg%d" % i, j, msg_len) for j in range(L)]
        order = sorted(range(L), key=lambda j: drbg(seed, b"disc%d" % i, j, 8))
        reqs.append({"msgs": msgs, "hdr": drbg(seed, b"hdr", i, 64), "ph": drbg(seed, b"ph", i, 64),
                     "di": sorted(order[:R]), "seed": drbg(seed, b"blind", i, 32)})
    return reqs


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_oracle_proof_verify(items, seconds_budget, threads):
    """Times the oracle's ProofVerify over a bounded sample on `threads` host threads."""
    sys.path.insert(0, str(ROOT))
    from oracle import oracle_ctypes as O
    O.lib()
    # probe the single-op cost to size the sample to ~seconds_budget of CPU work
    t0 = time.perf_counter()
    it = items[0]
    rc = O.proof_verify(it[0], it[1], it[2], it[3], it[4], it[5])
    assert rc == 0, "oracle rejected a GPU-generated proof"
    one = time.perf_counter() - t0
    sample = max(threads, int(seconds_budget * threads / max(one, 1e-4)))
    sample = min(sample, 20000)
    sample = (sample // threads) * threads or threads
    work = [items[i % len(items)] for i in range(sample)]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        rcs = list(ex.map(lambda x: O.proof_verify(x[0], x[1], x[2], x[3], x[4], x[5]), work))
    dt = time.perf_counter() - t0
    assert all(r == 0 for r in rcs)
    return sample / dt, sample, dt


def fixed_msm_section(pkg, rank):
    """C2: 4096 independent 12-term fixed-base MSMs (bases P1, Q1, H1..H10, scalars
    uniform mod r).  The autotuner rebuilds the resident table for window widths
    4..12 and keeps the fastest; e2e goes through the common-points ABI call."""
    rows, terms = 4096, 12
    seed = b"cubbs-bench-c2-%d" % rank
    scal = [(int.from_bytes(drbg(seed, b"s", i, 48), "big") % R_MOD).to_bytes(32, "big") for i in range(rows * terms)]
    ms_w, best_w = pkg.fixed_msm_autotune(b"".join(scal), rows, terms, 4, 20, steps=3)
    best_ms = ms_w[best_w - 4]
    g = json.loads((ROOT / "tests" / "golden" / "cfrg_bls12381_sha256.json").read_text())["generators"]
    gens = [bytes.fromhex(x) for x in [g["P1"], g["Q1"]] + g["MsgGenerators"]][:terms]
    call = pkg.prepared_common_points_call(gens, [scal[r * terms:(r + 1) * terms] for r in range(rows)])
    for _ in range(3):
        call()
    e2e = []
    for _ in range(5):
        t0 = time.perf_counter()
        out = call()
        e2e.append(time.perf_counter() - t0)
    assert all(c == 0 for c, _, _ in out)
    return {"workload": "4096 fixed-base G1 MSMs x 12 terms over [P1, Q1, H1..H10], affine out",
            "msms_per_s": round(rows / (best_ms / 1e3), 1), "kernel_ms": round(best_ms, 4),
            "window_sweep_ms": {str(w): round(ms, 4) for w, ms in zip(range(4, 21), ms_w)},
            "autotuned_window": best_w,
            "e2e_msms_per_s": round(rows / statistics.mean(e2e), 1)}


def uneven_msm_section(pkg, rank):
    """C4: 16384 variable-base MSMs with K ~ U{2..257} (points u*P1, scalars uniform
    mod r, one seed); thread-versus-warp mode, chunk length and window (4..12) per
    size class autotuned; the engine replayed as one CUDA graph (prep +
    persistent launch + reduction)."""
    n = 16384
    r = pkg.msm_uneven_bench(n_msms=n, k_min=2, k_max=257, seed=4 + rank, tune=True, warmup=3, steps=5)
    assert r["mismatch"] == 0, "uneven MSM engine disagrees with the per-term path"
    ms = statistics.mean(r["ms"])
    return {"workload": "16384 variable-base G1 MSMs, K ~ U{2..257}, points u*P1, scalars uniform mod r",
            "msms_per_s": round(n / (ms / 1e3), 1), "ms_per_batch": round(ms, 3),
            "decode_ms_all_points": round(r["decode_ms"], 3),
            "msms_per_s_with_decode": round(n / ((ms + r["decode_ms"]) / 1e3), 1),
            "autotuned": {"size_classes": ["K<=8", "K<=32", "K<=96", "K<=257"], "chunk_terms": r["chunk"],
                          "window_bits": r["window"],
                          "mode": ["warp" if m else "thread" for m in r["mode"]]},
            "checked_vs_per_term_glv": r["checked"], "l2": "flushed (256 MiB write) before each replay"}


def serving_section(pkg, rank):
    """C5: Poisson arrivals of a 40/40/10/10 Sign/Verify/ProofGen/ProofVerify mix,
    L ~ U{5,10,20,50,100,200}, disclosure ~ U[0.1, 0.9], 256 keypairs with their
    public-key lines device-resident; p50/p99 latency and ops/s of the serving queue
    (continuous batching) against plain fixed-size batches (256 requests, 2 ms)."""
    import random
    keys = json.loads((ROOT / "tests" / "golden" / "keypairs256.json").read_text())
    keys = [(bytes.fromhex(k["sk"]), bytes.fromhex(k["pk"])) for k in keys]
    rng = random.Random(1000 + rank)
    seed = b"cubbs-bench-c5-%d" % rank
    P = 2048
    plan = []
    for i in range(P):
        u = rng.random()
        op = pkg.OP_SIGN if u < 0.4 else pkg.OP_VERIFY if u < 0.8 else pkg.OP_PROOF_GEN if u < 0.9 else pkg.OP_PROOF_VERIFY
        L = rng.choice((5, 10, 20, 50, 100, 200))
        f = rng.uniform(0.1, 0.9)
        plan.append((op, L, max(1, round(f * L)), rng.randrange(256)))
    # signatures for everything that needs one, then proofs (this library, untimed)
    base = []
    for i, (op, L, R, kidx) in enumerate(plan):
        msgs = [drbg(seed, b"m%d" % i, j, 64) for j in range(L)]
        order = sorted(range(L), key=lambda j: drbg(seed, b"d%d" % i, j, 8))
        base.append({"msgs": msgs, "hdr": drbg(seed, b"h", i, 64), "ph": drbg(seed, b"p", i, 64),
                     "di": sorted(order[:R]), "seed": drbg(seed, b"b", i, 32), "sk": keys[kidx][0],
                     "pk": keys[kidx][1]})
    need = [i for i, (op, *_ ) in enumerate(plan) if op != pkg.OP_SIGN]
    sigs = pkg.sign_batch([(base[i]["sk"], base[i]["pk"], base[i]["hdr"], base[i]["msgs"]) for i in need])
    sig_of = {i: s for i, (_, s) in zip(need, sigs)}
    pv = [i for i, (op, *_ ) in enumerate(plan) if op == pkg.OP_PROOF_VERIFY]
    proofs = pkg.proof_gen_batch([(base[i]["pk"], sig_of[i], base[i]["hdr"], base[i]["ph"], base[i]["msgs"],
                                   base[i]["di"]) for i in pv], seeds=[base[i]["seed"] for i in pv])
    proof_of = {i: p for i, (_, p) in zip(pv, proofs)}
    pool = []
    for i, (op, L, R, _) in enumerate(plan):
        b = base[i]
        if op == pkg.OP_SIGN:
            pool.append((op, (b["sk"], b["pk"], b["hdr"], b["msgs"]), None))
        elif op == pkg.OP_VERIFY:
            pool.append((op, (b["pk"], sig_of[i], b["hdr"], b["msgs"]), None))
        elif op == pkg.OP_PROOF_GEN:
            pool.append((op, (b["pk"], sig_of[i], b["hdr"], b["ph"], b["msgs"], b["di"]), b["seed"]))
        else:
            pool.append((op, (b["pk"], proof_of[i], b["hdr"], b["ph"], [b["msgs"][j] for j in b["di"]], b["di"], L),
                         None))
    # warm the prepared state (256 keys' lines, generator tables) untimed
    res, _, _ = pkg.serve_replay(pool, [(i, 0) for i in range(P)], mode=pkg.SERVE_QUEUE)
    assert all(c == 0 for c, _, _ in res)
    assert all(v == 1 for (op, _, _), (c, v, _) in zip(pool, res) if op in (pkg.OP_VERIFY, pkg.OP_PROOF_VERIFY))
    out = []
    for rate in (5000, 20000, 50000, 100000, 200000):
        count = max(2000, min(40000, int(rate * 0.4)))
        t, schedule = 0.0, []
        for _ in range(count):
            t += rng.expovariate(rate)
            schedule.append((rng.randrange(P), int(t * 1e9)))
        row = {"rate_req_s": rate, "requests": count}
        for name, mode in (("served", pkg.SERVE_QUEUE), ("plain", pkg.SERVE_PLAIN)):
            res, lat, wall = pkg.serve_replay(pool, schedule, mode=mode, plain_batch=256, plain_timeout_us=2000)
            assert all(c == 0 for c, _, _ in res)
            lat_ms = sorted(x / 1e6 for x in lat)
            row[name] = {"p50_ms": round(lat_ms[len(lat_ms) // 2], 3),
                         "p99_ms": round(lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))], 3),
                         "ops_per_s": round(count / wall, 1)}
        out.append(row)
    return {"workload": "Poisson arrivals, 40/40/10/10 Sign/Verify/ProofGen/ProofVerify, L~U{5..200}, "
                        "disclosure~U[0.1,0.9], 256 device-resident keys; served = continuous batching "
                        "(4 slots, HBM budget 1 GiB), plain = batches of 256 or 2 ms, one at a time",
            "rates": out}


def serving_pv_section(pkg, rank, pv_reqs):
    """The spec comparison: ProofVerify at L = 100 with 50 of 100 messages
    disclosed, single requests under Poisson arrivals, served by the queue
    (continuous batching) and by the plain batched launch of the headline (batches
    of 1024 or 2 ms, one at a time).  Reports p50 / p99 latency and ops/s per rate,
    and for each mode the highest rate whose p99 stays within P99_BOUND_MS."""
    import random
    P99_BOUND_MS = 50.0
    REPEATS = 3
    rng = random.Random(2000 + rank)
    pool = [(pkg.OP_PROOF_VERIFY, r, None) for r in pv_reqs]
    res, _, _ = pkg.serve_replay(pool, [(i, 0) for i in range(len(pool))], mode=pkg.SERVE_QUEUE)  # warm
    assert all(c == 0 and v == 1 for c, v, _ in res)
    rows, best = [], {"served": None, "plain": None}
    for rate in (25000, 50000, 100000, 150000, 175000, 200000, 225000, 250000, 275000, 300000, 350000, 400000):
        count = max(4096, min(60000, int(rate * 0.2)))
        row = {"rate_req_s": rate, "requests": count, "repeats": REPEATS}
        runs = {"served": [], "plain": []}
        for rep in range(REPEATS):
            t, schedule = 0.0, []
            for _ in range(count):
                t += rng.expovariate(rate)
                schedule.append((rng.randrange(len(pool)), int(t * 1e9)))
            for name, mode in (("served", pkg.SERVE_QUEUE), ("plain", pkg.SERVE_PLAIN)):
                res, lat, wall = pkg.serve_replay(pool, schedule, mode=mode, plain_batch=1024,
                                                  plain_timeout_us=2000)
                assert all(c == 0 and v == 1 for c, v, _ in res)
                lat_ms = sorted(x / 1e6 for x in lat)
                runs[name].append((lat_ms[len(lat_ms) // 2], lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))],
                                   count / wall))
        for name in ("served", "plain"):
            p50s, p99s, opss = zip(*runs[name])
            med = lambda v: statistics.median(v)
            row[name] = {"p50_ms": round(med(p50s), 3), "p99_ms": round(med(p99s), 3),
                         "ops_per_s": round(med(opss), 1),
                         "p99_ms_min_max": [round(min(p99s), 3), round(max(p99s), 3)],
                         "ops_per_s_min_max": [round(min(opss), 1), round(max(opss), 1)]}
            if row[name]["p99_ms"] <= P99_BOUND_MS and (best[name] is None or
                                                        row[name]["ops_per_s"] > best[name]["ops_per_s"]):
                best[name] = {"rate_req_s": rate, **row[name]}
        rows.append(row)
    # matched p99: the served rate with the most ops/s whose median p99 is no
    # larger than the plain path's at its best rate within the bound
    matched = None
    if best["plain"] is not None:
        cap = best["plain"]["p99_ms"]
        cands = [r for r in rows if r["served"]["p99_ms"] <= cap]
        if cands:
            top = max(cands, key=lambda r: r["served"]["ops_per_s"])
            matched = {"plain_p99_ms": cap, "plain_ops_per_s": best["plain"]["ops_per_s"],
                       "served_rate_req_s": top["rate_req_s"], "served_p99_ms": top["served"]["p99_ms"],
                       "served_ops_per_s": top["served"]["ops_per_s"],
                       "served_over_plain": round(top["served"]["ops_per_s"] / best["plain"]["ops_per_s"], 3)}
    return {"workload": "ProofVerify L=100 x 64 B, 50 disclosed, Poisson arrivals of single requests; "
                        "served = continuous batching (4 slots, up to 1024 per batch), plain = batches of "
                        "1024 or 2 ms, one at a time (the headline batched launch); medians of %d runs per "
                        "rate" % REPEATS,
            "p99_bound_ms": P99_BOUND_MS, "best_within_p99_bound": best, "matched_p99": matched, "rates": rows}


def multi_key_pv_section(pkg, rank, L, R, args):
    """The headline ProofVerify batch spread over 64 keys (16 proofs per key, so
    every key is one aggregated group of 16): device-resident ops/s beside the
    single-key headline."""
    keys = json.loads((ROOT / "tests" / "golden" / "keypairs256.json").read_text())[:64]
    keys = [(bytes.fromhex(k["sk"]), bytes.fromhex(k["pk"])) for k in keys]
    n = args.batch
    reqs = make_requests(n, L, R, 64, b"cubbs-bench-mk-%d" % rank)
    sigs = pkg.sign_batch([(keys[i % 64][0], keys[i % 64][1], r["hdr"], r["msgs"]) for i, r in enumerate(reqs)])
    assert all(c == 0 for c, _ in sigs)
    proofs = pkg.proof_gen_batch([(keys[i % 64][1], s, r["hdr"], r["ph"], r["msgs"], r["di"])
                                  for i, (r, (_, s)) in enumerate(zip(reqs, sigs))], seeds=[r["seed"] for r in reqs])
    assert all(c == 0 for c, _ in proofs)
    pv = [(keys[i % 64][1], p, r["hdr"], r["ph"], [r["msgs"][j] for j in r["di"]], r["di"], L)
          for i, (r, (_, p)) in enumerate(zip(reqs, proofs))]
    ms, _, res, stages = pkg.bench_device_steps(pkg.OP_PROOF_VERIFY, pv, args.warmup, args.steps)
    assert all(c == 0 and v == 1 for c, v in res)
    step = statistics.mean(ms)
    return {"workload": "the headline batch (%d proofs, L=%d, %d disclosed) over 64 keys, 16 proofs per key" %
                        (n, L, R),
            "ops_per_s": round(n / (step / 1e3), 2), "ms_per_step": round(step, 3),
            "stages_ms": {k: round(v, 3) for k, v in stages}}


def reference_arm(args):
    """The reference's CPU implementation of the path (oracle port), rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT))
    from oracle import oracle_ctypes as O
    O.lib()
    threads = os.cpu_count() or 1
    reqs = make_requests(threads * 2, args.L, args.R, 64, b"cubbs-bench-ref")
    # build the sample with the oracle itself: sign, then prove (untimed)
    def prep(r):
        sig, _, _ = O.sign(SK, PK, r["hdr"], r["msgs"])
        proof = O.proof_gen(PK, sig, r["hdr"], r["ph"], r["msgs"], r["di"], seed=r["seed"])
        return (PK, proof, r["hdr"], r["ph"], [r["msgs"][j] for j in r["di"]], r["di"])
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        items = list(ex.map(prep, reqs))
    per_step = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            rcs = list(ex.map(lambda x: O.proof_verify(*x), items))
        dt = time.perf_counter() - t0
        assert all(r == 0 for r in rcs)
        if k >= args.warmup:
            per_step.append(dt)
    ms = 1e3 * statistics.mean(per_step)
    value = len(items) / (ms / 1e3)
    line = {"impl": "reference", "metric": "BBS ProofVerify ops/sec at L=100 (1 GB300)", "value": round(value, 2),
            "unit": "ops/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32 (exact mod p / mod r)", "data": "synthetic (seeded DRBG)",
            "config": {"workload": "BBS ProofVerify, L=100 x 64 B, 50 disclosed, CPU sample of %d proofs" % len(items),
                       "L": args.L, "disclosed": args.R, "sample_proofs": len(items)},
            "cpu_baseline": {"value": round(value, 2), "unit": "ops/s", "cores": threads, "kind": "port",
                             "sample": "%d ProofVerify ops per step on %d threads (C++ oracle restating the "
                                       "reference Rust CPU path)" % (len(items), threads)},
            "e2e": {"value": round(value, 2), "unit": "ops/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="cubbs")
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--L", type=int, default=100)
    ap.add_argument("--R", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true", help="headline only (no C2/C5 sections)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        reference_arm(args)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    os.environ["CUBBS_BBS_DEVICE"] = str(local)
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    pkg = load_package()
    pkg.build()
    kind, hw = pkg.backend_info()
    assert kind == pkg.BACKEND_KIND_CUDA and hw == 1

    # ---------------- workload (untimed): signatures and proofs from this library
    n, L, R = args.batch, args.L, args.R
    seed = b"cubbs-bench-%d" % rank
    reqs = make_requests(n, L, R, 64, seed)
    t_cold = time.perf_counter()  # the first call builds the prepared state (generators, table, key lines)
    sigs = pkg.sign_batch([(SK, PK, r["hdr"], r["msgs"]) for r in reqs])
    cold_s = time.perf_counter() - t_cold
    assert all(c == 0 for c, _ in sigs)
    pg_reqs = [(PK, s, r["hdr"], r["ph"], r["msgs"], r["di"]) for r, (_, s) in zip(reqs, sigs)]
    proofs = pkg.proof_gen_batch(pg_reqs, seeds=[r["seed"] for r in reqs])
    assert all(c == 0 for c, _ in proofs)
    pv_reqs = [(PK, p, r["hdr"], r["ph"], [r["msgs"][j] for j in r["di"]], r["di"], L)
               for r, (_, p) in zip(reqs, proofs)]

    tera_imad, giga_fpmul = pkg.int_peaks()
    table_w = pkg.table_window()  # chosen for the 102 generators of L = 100
    table_gens = max(64, 1 << (L + 1).bit_length())  # the library keeps a power of two, at least 64
    prepared = {"table_window": table_w, "table_generators": table_gens,
                "table_bytes": table_gens * (255 // table_w + 1) * (1 << (table_w - 1)) * 96,
                "first_call_s": round(cold_s, 3),
                "first_call": "Sign of the 1024-item batch on a fresh process: generators by hash_to_curve, "
                              "the fixed-base table, the key's Miller lines, then the batch"}
    part_sms = pkg.sm_partition()
    var_sms = pkg.sm_partition_var()[0]

    # ---------------- timed: device-resident ProofVerify (headline) + ProofGen
    def barrier():
        if dist is not None:
            dist.barrier()

    barrier()
    with ClockSampler(local) as clk:
        pv_ms, pv_launch, pv_res, pv_stages = pkg.bench_device_steps(pkg.OP_PROOF_VERIFY, pv_reqs, args.warmup,
                                                                     args.steps)
    barrier()
    assert all(c == 0 and v == 1 for c, v in pv_res), "ProofVerify rejected a valid proof"
    pg_ms, pg_launch, pg_res, pg_stages = pkg.bench_device_steps(pkg.OP_PROOF_GEN, pg_reqs, args.warmup,
                                                                 args.steps, seeds=[r["seed"] for r in reqs])
    assert all(c == 0 for c, _ in pg_res)
    sv_reqs = [(SK, PK, r["hdr"], r["msgs"][:10]) for r in reqs[:64]]
    sg_ms, _, _, _ = pkg.bench_device_steps(pkg.OP_SIGN, sv_reqs, args.warmup, args.steps)
    vsigs = pkg.sign_batch(sv_reqs)
    vf_ms, _, vf_res, _ = pkg.bench_device_steps(pkg.OP_VERIFY, [(PK, s, r[2], r[3]) for r, (_, s) in
                                                                 zip(sv_reqs, vsigs)], args.warmup, args.steps)
    assert all(c == 0 and v == 1 for c, v in vf_res)

    # ---------------- e2e: the C ABI with host buffers, transfers inside the timed region.
    # The caller's item structs (its own data) are built once; each timed step is one
    # synchronous cubbs_bbs_gpu_proof_verify_batch_v2 call: packing, H2D, the device
    # pipeline, D2H and result mapping.
    call = pkg.prepared_call(pkg.OP_PROOF_VERIFY, pv_reqs)
    for _ in range(args.warmup):
        call()
    barrier()
    e2e = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out = call()
        e2e.append(time.perf_counter() - t0)
    barrier()
    assert all(c == 0 and v for c, v in out)
    h2d, d2h = pkg.last_transfer_bytes()

    # ---------------- C2: 4096 fixed-base MSMs of 12 terms over [P1, Q1, H1..H10];
    # the window width of the resident table is swept by the autotuner
    c2 = fixed_msm_section(pkg, rank) if not args.quick else None

    # ---------------- C4: 16384 uneven variable-base MSMs, persistent launch in a CUDA graph
    c4 = uneven_msm_section(pkg, rank) if not args.quick else None

    # ---------------- C5: serving queue vs plain batches under Poisson arrivals
    c5 = serving_section(pkg, rank) if not args.quick else None
    c5_pv = serving_pv_section(pkg, rank, pv_reqs) if not args.quick else None
    c3_mk = multi_key_pv_section(pkg, rank, L, R, args) if not args.quick else None

    pv_step = statistics.mean(pv_ms)
    e2e_step = statistics.mean(e2e) * 1e3
    if dist is not None:
        import torch
        t = torch.tensor([pv_step, e2e_step], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        pv_step, e2e_step = float(t[0]), float(t[1])
    value = world * n / (pv_step / 1e3)
    e2e_value = world * n / (e2e_step / 1e3)

    # ---------------- roofline: dominant stage of the ProofVerify pipeline vs the IMAD peak
    # (the pairing kernel runs on a second stream beside the MSMs; its own
    # event-timed duration is the "pairing_kernel" entry)
    modelled = [s for s in pv_stages if s[0] in MODEL_M["proof_verify"]] or pv_stages
    stage = max(modelled, key=lambda s: s[1])
    model = MODEL_M["proof_verify"].get(stage[0])
    roof = None
    if model:
        achieved = n * model * IMAD_PER_M / (stage[1] / 1e3) / 1e12
        traffic = TRAFFIC_BYTES.get(stage[0])
        if traffic is not None and (n, L) != (1024, 100):
            traffic = None  # measured for the 1024-proof, L = 100 workload only
        roof = {"bound": "imad", "kernel": stage[0], "achieved": round(achieved, 3), "peak": round(tera_imad, 3),
                "unit": "T IMAD/s (32-bit integer multiply-add)", "frac": round(achieved / tera_imad, 4),
                "traffic": round(traffic) if traffic else None,
                "traffic_unit": "bytes per launch (ncu capture of this step; the fixed-base MSM's with the table at "
                                "window 14, scaled to window 20)",
                "peak_source": "measured in this run (k_imad_peak, 16 independent mad.lo chains)",
                "partition_sms": var_sms if stage[0] == "var_mul" and var_sms else None,
                "frac_of_partition": round(achieved / tera_imad * (part_sms[0] + part_sms[1]) / var_sms, 4)
                if stage[0] == "var_mul" and var_sms else None,
                "model_m_per_op": model, "stage_ms": round(stage[1], 3)}
    whole = n * MODEL_M["proof_verify"]["total"] * IMAD_PER_M / (pv_step / 1e3) / 1e12

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        items = [(PK, p[1], p[2], p[3], p[4], p[5]) for p in pv_reqs[:64]]
        v, sample, dt = cpu_oracle_proof_verify(items, args.cpu_seconds, threads)
        cpu = {"value": round(v, 2), "unit": "ops/s", "cores": threads, "kind": "port",
               "sample": "%d ProofVerify ops (L=100, 50 disclosed) in %.1f s on %d threads; C++ oracle "
                         "restating the reference Rust CPU path" % (sample, dt, threads)}

    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": "BBS ProofVerify ops/sec at L=100 (1 GB300)",
            "value": round(value, 2), "unit": "ops/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(pv_step, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32 (exact mod p / mod r)",
            "data": "synthetic (seeded DRBG; signatures/proofs generated by this library)",
            "config": {"workload": "BBS ProofGen+ProofVerify, L=100 x 64 B, 50 disclosed, 1024 proofs per batch",
                       "batch": n, "L": L, "disclosed": R, "l2": "flushed (256 MiB write) between timed steps",
                       "fixed_base_window": table_w, "prepared_state": prepared,
                       "sm_partition": {"pairing_check": part_sms[0], "rest": part_sms[1],
                                        "var_terms": pkg.sm_partition_var()[0],
                                        "var_terms_status": pkg.sm_partition_var()[1],
                                        "status": part_sms[2]},
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "per_op_ops_per_s": {
                "proof_verify_L100": round(value / world, 2),
                "proof_gen_L100": round(n / (statistics.mean(pg_ms) / 1e3), 2),
                "sign_L10_batch64": round(len(sv_reqs) / (statistics.mean(sg_ms) / 1e3), 2),
                "verify_L10_batch64": round(len(sv_reqs) / (statistics.mean(vf_ms) / 1e3), 2)},
            "stages_ms": {"proof_verify": {k: round(v, 3) for k, v in pv_stages},
                          "proof_gen": {k: round(v, 3) for k, v in pg_stages}},
            "roofline": roof,
            "roofline_whole_op": {"achieved_t_imad": round(whole, 3), "frac": round(whole / tera_imad, 4),
                                  "model_m_per_op": MODEL_M["proof_verify"]["total"]},
            "int_peaks": {"t_imad_per_s": round(tera_imad, 3), "g_fp_mul_per_s": round(giga_fpmul, 2)},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 2), "unit": "ops/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": pv_launch * args.steps,
            "clocks": clocks,
            "fixed_base_msm_c2": c2,
            "uneven_msm_c4": c4,
            "serving_c5": c5,
            "serving_pv_L100": c5_pv,
            "proof_verify_L100_64_keys": c3_mk,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
