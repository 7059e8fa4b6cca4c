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
