"""Layer-by-layer device checks (Fp, G1 decode, GLV scalar mul) against the oracle."""
import pytest

from helpers import drbg, scalar

pytestmark = pytest.mark.gpu


def rand_fp(oracle, label, n):
    return [(int.from_bytes(drbg(b"fp", label, i, 64), "big") % oracle.P_MOD).to_bytes(48, "big") for i in range(n)]


def test_fp_mul(gpu, oracle):
    a = rand_fp(oracle, b"a", 64) + [(oracle.P_MOD - 1).to_bytes(48, "big"), bytes(48)]
    b = rand_fp(oracle, b"b", 64) + [(oracle.P_MOD - 1).to_bytes(48, "big"), (1).to_bytes(48, "big")]
    got = gpu.fp_op_for_test(0, a, b)
    assert [g[1] for g in got] == [oracle.fp_mul(x, y) for x, y in zip(a, b)]


def test_fp_mul_carry_save(gpu, oracle):
    """The carry-save product (fp_mul) equals the CIOS product and the oracle, edge operands included."""
    edge = [oracle.P_MOD - 1, oracle.P_MOD - 2, 1, 0, 2, (1 << 380) % oracle.P_MOD, (1 << 352) - 1]
    a = rand_fp(oracle, b"csa", 2048) + [x.to_bytes(48, "big") for x in edge for _ in edge]
    b = rand_fp(oracle, b"csb", 2048) + [y.to_bytes(48, "big") for _ in edge for y in edge]
    cs = gpu.fp_op_for_test(0, a, b)
    cios = gpu.fp_op_for_test(4, a, b)
    assert [g[1] for g in cs] == [g[1] for g in cios]
    assert [g[1] for g in cs] == [oracle.fp_mul(x, y) for x, y in zip(a, b)]


def test_fp_inv_sqrt(gpu, oracle):
    a = rand_fp(oracle, b"inv", 16)
    inv = gpu.fp_op_for_test(1, a, a)
    one = (1).to_bytes(48, "big")
    for x, (_, xi) in zip(a, inv):
        assert oracle.fp_mul(x, xi) == one
    sq = [oracle.fp_mul(x, x) for x in a]
    roots = gpu.fp_op_for_test(2, sq, sq)
    for s, (st, r) in zip(sq, roots):
        assert st == 0 and oracle.fp_mul(r, r) == s


def test_fp_inv_vartime_matches_fermat(gpu, oracle):
    a = rand_fp(oracle, b"vinv", 48) + [(1).to_bytes(48, "big"), (oracle.P_MOD - 1).to_bytes(48, "big"),
                                        (2).to_bytes(48, "big"), bytes(48)]
    fermat = gpu.fp_op_for_test(1, a, a)
    binary = gpu.fp_op_for_test(3, a, a)
    assert [r for _, r in binary] == [r for _, r in fermat]
    assert binary[-1][1] == bytes(48)


def test_g1_decode_and_mul(gpu, oracle):
    p1, gens = oracle.generators(8)
    pts = [p1] + gens
    ks = [scalar(b"g1t", b"k", i) for i in range(len(pts))]
    got = gpu.g1_op_for_test(pts, ks)
    mults = [2, 3, 3, 4, 5, 4, 18, 0xD201000000010000, 0, 0xD201000000010000, 0xD201000000010000, 0xD201000000010000]
    report = []
    for p, k, (st, xy, kp, diag, chain) in zip(pts, ks, got):
        want = [oracle.g1_mul(p, m.to_bytes(32, "big")) for m in mults]
        want[8] = diag[8]  # unused slot
        bad = [j for j in range(len(mults)) if diag[j] != want[j]]
        wchain = [oracle.g1_mul(p, (2 ** (j + 1) % oracle.R_MOD).to_bytes(32, "big")) for j in range(64)]
        bad_chain = [j + 1 for j in range(64) if chain[j] != wchain[j]]
        report.append((st, bad, bad_chain[:5], kp == oracle.g1_mul(p, k), xy == oracle.g1_decompress(p)))
    print("G1 REPORT", report)
    assert all(r == (0, [], [], True, True) for r in report), report


def test_h2s_over_scalars(gpu, oracle):
    import ctypes
    fn = gpu.lib().cubbs_bbs_gpu_h2s_scalars_for_test_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p]
    for n in (1, 2, 3, 12):
        ss = [scalar(b"h2ss", b"s", i) for i in range(n)]
        blob = b"".join(ss)
        out = ctypes.create_string_buffer(32)
        assert fn(2, blob, n, ctypes.cast(out, ctypes.c_void_p)) == 0
        assert out.raw == oracle.hash_to_scalar(blob, gpu.H2S_DST), n


def test_disclosed_pairs_hash(gpu, oracle):
    import ctypes
    import struct
    fn = gpu.lib().cubbs_bbs_gpu_pairs_h2s_for_test_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32,
                   ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p]
    for R in (1, 2, 5):
        idx = [3 * k + 1 for k in range(R)]
        ms = [scalar(b"pairs", b"m", k) for k in range(R)]
        blob = b"\x01\x02\x03\x04" * 5 + b"".join(struct.pack("<I", i) for i in idx) + b"tail"
        out = ctypes.create_string_buffer(32)
        echo = (ctypes.c_uint32 * R)()
        assert fn(2, blob, len(blob), 20, R, b"".join(ms), ctypes.cast(out, ctypes.c_void_p),
                  ctypes.cast(echo, ctypes.c_void_p)) == 0
        stream = R.to_bytes(8, "big") + b"".join(i.to_bytes(8, "big") + m for i, m in zip(idx, ms))
        assert list(echo) == idx
        assert out.raw == oracle.hash_to_scalar(stream, gpu.H2S_DST), R


def test_proof_debug_record(gpu, oracle, golden):
    import ctypes
    c = golden["proof"][0]
    h = bytes.fromhex
    msgs = [h(m) for m in c["messages"]]
    req = (h(c["signerPublicKey"]), h(c["signature"]), h(c["header"]), h(c["presentationHeader"]), msgs,
           c["disclosedIndexes"])
    gpu.proof_gen_batch([req], seeds=[oracle.SEED_MOCKED_SCALAR])
    rec = ctypes.create_string_buffer(256)
    fn = gpu.lib().cubbs_bbs_gpu_last_debug_record_for_test_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p]
    assert fn(ctypes.cast(rec, ctypes.c_void_p)) == 0
    r = rec.raw
    tr = c["trace"]
    got = {"T1": r[0:48].hex(), "T2": r[48:96].hex(), "domain": r[96:128].hex(), "challenge": r[128:160].hex(),
           "R": int.from_bytes(r[160:164], "little"), "idx0": int.from_bytes(r[164:168], "little"),
           "m0": r[180:212].hex()}
    want = {"T1": tr["T1"], "T2": tr["T2"], "domain": tr["domain"], "challenge": tr["challenge"], "R": 1, "idx0": 0,
            "m0": oracle.hash_to_scalar(msgs[0], oracle.MAP_DST).hex()}
    print("DEBUG RECORD", {k: (got[k] == want[k]) for k in got}, got)
    assert got == want
