"""The allocation-free G1 MSM entry point (cubbs_bbs_gpu_g1_msm_noalloc_v2)
against the arena-backed cubbs_bbs_gpu_g1_msm_batch_v2, through the C ABI.

Collected last so it also runs after every other GPU test in the same process;
it passes on its own in a fresh process too.  Integer work: bit-exact."""
import pytest

from helpers import scalar

pytestmark = pytest.mark.gpu


def rand_points(oracle, seed, n):
    p1, _ = oracle.generators(1)
    return [oracle.g1_mul(p1, scalar(seed, b"pt", i)) for i in range(n)]


def rand_scalars(seed, n):
    return [scalar(seed, b"k", i) for i in range(n)]


def test_two_calls_in_a_row_match_batch_entry(gpu, oracle):
    # the scratch array is reused: the second call must not see the first one's data
    first = (rand_points(oracle, b"na-1", 37), rand_scalars(b"na-1", 37))
    second = (rand_points(oracle, b"na-2", 5), rand_scalars(b"na-2", 5))
    got = [gpu.g1_msm_noalloc(*first), gpu.g1_msm_noalloc(*second)]
    want = gpu.g1_msm_batch([first, second])
    assert [(rc, code, p) for rc, code, p in got] == [(0, c, p) for c, p in want]
    assert all(c == 0 for c, _ in want)
    assert got[0][2] == oracle.g1_msm(*first)
    assert got[1][2] == oracle.g1_msm(*second)


def test_maximum_term_count(gpu, oracle):
    n = gpu.NOALLOC_MSM_MAX_TERMS
    _, gens = oracle.generators(n)
    scs = rand_scalars(b"na-max", n)
    rc, code, out = gpu.g1_msm_noalloc(gens, scs)
    (bcode, bout), = gpu.g1_msm_batch([(gens, scs)])
    assert (rc, code, out) == (0, bcode, bout) and bcode == 0


def test_over_limit_is_rejected(gpu):
    n = gpu.NOALLOC_MSM_MAX_TERMS + 1
    rc, code, _ = gpu.g1_msm_noalloc([bytes(48)] * n, [bytes(32)] * n)
    assert rc == gpu.ERR_NOALLOC_LIMIT and code == gpu.ERR_NOALLOC_LIMIT


def test_empty_identity_and_bad_inputs_match_batch_entry(gpu, oracle):
    pts = rand_points(oracle, b"na-edge", 4)
    scs = rand_scalars(b"na-edge", 4)
    ident = bytes([0xC0]) + bytes(47)
    off_curve = bytes([pts[1][0] ^ 0x01]) + pts[1][1:]
    r_mod = (0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001).to_bytes(32, "big")
    cases = [([], []),
             ([ident] + pts[1:], scs),
             (pts, [bytes(32)] * 4),
             ([pts[0], off_curve] + pts[2:], scs),
             (pts, scs[:3] + [r_mod]),
             (pts, scs)]
    want = gpu.g1_msm_batch(cases)
    for case, (bcode, bout) in zip(cases, want):
        rc, code, out = gpu.g1_msm_noalloc(*case)
        assert rc == 0 and code == bcode
        if code == 0:
            assert out == bout
    assert [c for c, _ in want] == [0, 0, 0, gpu.ERR_INVALID_INPUT, gpu.ERR_INVALID_INPUT, 0]
    assert want[0][1] == ident and want[2][1] == ident


NO_ALLOC_CHILD = r"""
import ctypes, json, sys
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
from tests.conftest import load_package
from oracle import oracle_ctypes as O
from helpers import scalar
pkg = load_package()
pkg.build()
pkg.lib()  # loads libcudart through the library's own dependency
cudart = ctypes.CDLL("libcudart.so.13")
free, total = ctypes.c_size_t(), ctypes.c_size_t()
def free_bytes():
    assert cudart.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value
p1, _ = O.generators(1)
pts = [O.g1_mul(p1, scalar(b"na-mem", b"pt", i)) for i in range(64)]
scs = [scalar(b"na-mem", b"k", i) for i in range(64)]
first = pkg.g1_msm_noalloc([], [])  # set-up call with zero terms
before = free_bytes()
outs = [pkg.g1_msm_noalloc(pts[:n], scs[:n]) for n in (1, 37, 64, 2, 64)]
after = free_bytes()
print(json.dumps({"first": list(first[:2]), "codes": [o[:2] for o in outs], "before": before, "after": after,
                  "match": outs[2][2] == O.g1_msm(pts, scs)}))
"""


def test_no_device_allocation_after_set_up():
    """In a fresh process: a set-up call with zero terms, then calls of 1 to 64
    terms; the device's free memory (cudaMemGetInfo) does not move, so no call
    after the set-up allocated device memory (or grew the driver's local-memory
    reservation)."""
    import json
    import os
    import pathlib
    import subprocess
    import sys
    root = pathlib.Path(__file__).resolve().parents[1]
    out = subprocess.run([sys.executable, "-c", NO_ALLOC_CHILD, str(root)], capture_output=True, text=True,
                         timeout=600, env=dict(os.environ))
    assert out.returncode == 0, out.stderr[-3000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["first"] == [0, 0] and all(c == [0, 0] for c in res["codes"]) and res["match"]
    assert res["after"] == res["before"], res
