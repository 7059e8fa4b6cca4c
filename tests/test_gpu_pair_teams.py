"""Pairing checks on two-warp teams (64-lane phase tables) against one-warp
teams: the per-program cycles of a lone team, and Verify / ProofVerify
verdicts with either width equal to the oracle's.  The width is read at
library start, so the one-warp run is a child process with
CUBBS_BBS_PAIR_TEAM=32."""
import json
import os
import pathlib
import pickle
import subprocess
import sys
import tempfile

import pytest

from helpers import keypair, messages
from tests.test_gpu_parity import _pv_items

pytestmark = pytest.mark.gpu

ROOT = pathlib.Path(__file__).resolve().parents[1]

CHILD = r"""
import json, pickle, sys
sys.path.insert(0, sys.argv[1])
from tests.conftest import load_package
pkg = load_package()
pkg.build()
vf, pv = pickle.load(open(sys.argv[2], "rb"))
print(json.dumps({"verify": [bool(v) for _, v in pkg.verify_batch(vf)],
                  "proof_verify": [bool(v) for _, v in pkg.proof_verify_batch(pv)]}))
"""


def test_probe_both_widths(gpu):
    """Programs whose phases hold more than 32 products (the Miller steps and
    the Fp12 products) take fewer cycles on a two-warp team; the cyclotomic
    squaring (18 products) gains nothing."""
    narrow, wide = gpu.pairing_probe(), gpu.pairing_probe(wide=True)
    assert set(narrow) == set(wide) and all(v > 0 for v in narrow.values()) and all(v > 0 for v in wide.values())
    for prog in ("DBL1", "DBL", "MUL_F_F_X", "MUL_R_R_T"):
        assert wide[prog] < narrow[prog], (prog, wide[prog], narrow[prog])


def _verify_items(oracle, seed, n, bad):
    sk, pk = keypair(oracle, seed)
    items = []
    for i in range(n):
        msgs = messages(seed, i, 5, 32)
        sig = oracle.sign(sk, pk, b"h", msgs)[0]
        if i in bad:
            msgs = msgs[:-1] + [msgs[-1] + b"!"]
        items.append((pk, sig, b"h", msgs))
    return items


def test_verdicts_equal_with_either_width(gpu, oracle):
    """Verify (small batch: one split check per item; 160 items: a key group with
    failing items and its fallback) and ProofVerify (a failing group and its
    fallback): two-warp teams in this process, one-warp teams in a child."""
    vf = _verify_items(oracle, b"teams-v", 20, {3, 11}) + _verify_items(oracle, b"teams-w", 140, {0, 77})
    pv = _pv_items(oracle, b"teams-p", 130, 6, fake={9, 100})
    want_vf = [oracle.verify(pk, sig, h, m) == 0 for pk, sig, h, m in vf]
    want_pv = [oracle.proof_verify(pk, pr, hd, ph, dm, di) == 0 for pk, pr, hd, ph, dm, di, _ in pv]
    assert want_vf.count(False) == 4 and want_pv.count(False) == 2
    assert [v for _, v in gpu.verify_batch(vf[:20])] == want_vf[:20]
    assert [v for _, v in gpu.verify_batch(vf)] == want_vf
    assert [v for _, v in gpu.proof_verify_batch(pv)] == want_pv
    with tempfile.NamedTemporaryFile(suffix=".pkl", delete=False) as f:
        pickle.dump((vf, pv), f)
        path = f.name
    try:
        env = dict(os.environ, CUBBS_BBS_PAIR_TEAM="32")
        out = subprocess.run([sys.executable, "-c", CHILD, str(ROOT), path], env=env, capture_output=True,
                             text=True, timeout=600)
    finally:
        os.unlink(path)
    assert out.returncode == 0, out.stderr[-2000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["verify"] == want_vf and res["proof_verify"] == want_pv
