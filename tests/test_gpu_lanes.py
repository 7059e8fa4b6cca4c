"""The variable-base terms and the subgroup check on 1, 2, 4 and 8 lanes per
job (CUBBS_BBS_VAR_LANES, read once per process, so each setting runs in a child
process): G1 MSMs of the general route, ProofVerify verdicts (valid, tampered
and outside-G1 proofs) and ProofGen bytes all equal the oracle's."""
import json
import os
import pathlib
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = pathlib.Path(__file__).resolve().parents[1]

CHILD = r"""
import json, sys
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
from tests.conftest import load_package
from oracle import oracle_ctypes as O
from helpers import disclosed_subset, drbg, keypair, messages, scalar
from tests.test_gpu_parity import _on_curve_outside_g1
pkg = load_package(); pkg.build()
p1, _ = O.generators(1)
msms = []
for i in range(6):
    K = [1, 2, 5, 17, 40, 3][i]
    pts = [O.g1_mul(p1, scalar(b"lanes", b"pt%d" % i, k)) for k in range(K)]
    scs = [scalar(b"lanes", b"k%d" % i, k) for k in range(K)]
    if i == 3: pts[2] = bytes([0xC0]) + bytes(47)
    if i == 5: scs = [bytes(32), (1).to_bytes(32, "big"),
                      (0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000000).to_bytes(32, "big")]
    msms.append((pts, scs))
msm_ok = pkg.g1_msm_batch(msms) == [(0, O.g1_msm(p, s)) for p, s in msms]
sk, pk = keypair(O, b"lanes")
items, gen_reqs, seeds = [], [], []
for i in range(8):
    ms = messages(b"lanes", i, 12, 32)
    sig = O.sign(sk, pk, b"h", ms)[0]
    di = disclosed_subset(b"lanes", i, 12, 4)
    gen_reqs.append((pk, sig, b"h", b"p", ms, di))
    seeds.append(drbg(b"lanes", b"seed", i, 32))
gen = pkg.proof_gen_batch(gen_reqs, seeds=seeds)
pg_ok = all(c == 0 and p == O.proof_gen(*r, seed=s) for (c, p), r, s in zip(gen, gen_reqs, seeds))
for (pk_, sig, hd, ph, ms, di), (_, proof) in zip(gen_reqs, gen):
    items.append((pk_, proof, hd, ph, [ms[j] for j in di], di, 12))
bad = items[0][1]
items.append(items[1][:3] + (b"p2",) + items[1][4:])
items.append(items[2][:1] + (_on_curve_outside_g1(O, b"lanes") + bad[48:],) + items[2][2:])
want = [O.proof_verify(*it[:6]) == 0 for it in items]
pv_ok = [v for _, v in pkg.proof_verify_batch(items)] == want and want.count(False) == 2
print(json.dumps({"msm": msm_ok, "proof_gen": pg_ok, "proof_verify": pv_ok}))
"""


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_lane_modes_match_oracle(lanes):
    env = dict(os.environ, CUBBS_BBS_VAR_LANES=str(lanes))
    out = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], env=env, capture_output=True, text=True,
                         timeout=900)
    assert out.returncode == 0, out.stderr[-3000:]
    assert json.loads(out.stdout.strip().splitlines()[-1]) == {"msm": True, "proof_gen": True, "proof_verify": True}
