"""The SM partition of ProofVerify (two green contexts: the aggregation chain on a
few SMs of its own, every other kernel on the rest).  The partition is read at
library start, so the run without it is a child process with
CUBBS_BBS_SM_PARTITION=0; both runs must give the oracle's verdicts."""
import json
import os
import pathlib
import pickle
import subprocess
import sys
import tempfile

import pytest

from tests.test_gpu_parity import _pv_items

ROOT = pathlib.Path(__file__).resolve().parents[1]

CHILD = r"""
import json, pickle, sys
sys.path.insert(0, sys.argv[1])
from tests.conftest import load_package
pkg = load_package()
pkg.build()
items = pickle.load(open(sys.argv[2], "rb"))
print(json.dumps({"partition": list(pkg.sm_partition()),
                  "verdicts": [bool(v) for _, v in pkg.proof_verify_batch(items)]}))
"""


@pytest.mark.gpu
def test_partition_in_effect(gpu):
    """On GB300 (152 SMs) the split is 16 + 136; the driver builds partitions in
    multiples of 8 SMs."""
    small, rest, status = gpu.sm_partition()
    assert status == 0, f"SM partition off (status {status})"
    assert small == 16 and rest > small and small % 8 == 0


@pytest.mark.gpu
def test_proof_verify_same_without_partition(gpu, oracle):
    """A batch with a failing group (per-item fallback), a passing group and
    ungrouped items: verdicts with and without the partition equal the oracle's."""
    items = _pv_items(oracle, b"part-a", 130, 6, fake={7, 99}) + _pv_items(oracle, b"part-b", 20, 6) + \
        _pv_items(oracle, b"part-c", 5, 6, fake={2})
    want = [oracle.proof_verify(pk, pr, hd, ph, dm, di) == 0 for pk, pr, hd, ph, dm, di, _ in items]
    assert want.count(False) == 3
    got = [v for _, v in gpu.proof_verify_batch(items)]
    assert got == want
    with tempfile.NamedTemporaryFile(suffix=".pkl", delete=False) as f:
        pickle.dump(items, f)
        path = f.name
    try:
        env = dict(os.environ, CUBBS_BBS_SM_PARTITION="0")
        out = subprocess.run([sys.executable, "-c", CHILD, str(ROOT), path], env=env, capture_output=True,
                             text=True, timeout=600)
    finally:
        os.unlink(path)
    assert out.returncode == 0, out.stderr[-2000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["partition"][:2] == [0, 0] and res["partition"][2] == 1
    assert res["verdicts"] == want
