"""ctypes binding of the CPU oracle (test infrastructure only).

Loaded by tests/, the smoke entry and the CPU-baseline leg of bench.py, always
as the checker.  The GPU library never imports this module.
"""
import ctypes
import os
import pathlib
import subprocess
import threading

_HERE = pathlib.Path(__file__).resolve().parent
_LIB_PATH = _HERE / "build" / "libbbs_oracle.so"
_LOCK = threading.Lock()
_LIB = None

API_ID = b"BBS_BLS12381G1_XMD:SHA-256_SSWU_RO_H2G_HM2S_"
MAP_DST = API_ID + b"MAP_MSG_TO_SCALAR_AS_HASH_"
H2S_DST = API_ID + b"H2S_"
MOCKED_SCALAR_DST = API_ID + b"MOCK_RANDOM_SCALARS_DST_"
SEED_MOCKED_SCALAR = b"3.141592653589793238462643383279"
# ciphersuites (crates/cubbs-bbs-protocol/src/bbsplus/ciphersuites.rs:49-79)
SUITE_SHA256, SUITE_SHAKE256 = 0, 1
API_IDS = {SUITE_SHA256: API_ID, SUITE_SHAKE256: b"BBS_BLS12381G1_XOF:SHAKE-256_SSWU_RO_H2G_HM2S_"}


def suite_dsts(suite: int):
    """(map-to-scalar DST, hash-to-scalar DST, mocked-scalar DST) of a suite."""
    a = API_IDS[suite]
    return a + b"MAP_MSG_TO_SCALAR_AS_HASH_", a + b"H2S_", a + b"MOCK_RANDOM_SCALARS_DST_"

_u8p = ctypes.POINTER(ctypes.c_uint8)
_szp = ctypes.POINTER(ctypes.c_size_t)


def build() -> pathlib.Path:
    """Compile the oracle with its Makefile (a few seconds)."""
    subprocess.run(["make", "-s", "-C", str(_HERE)], check=True)
    return _LIB_PATH


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            if not _LIB_PATH.exists():
                build()
            _LIB = ctypes.CDLL(str(_LIB_PATH))
            _declare(_LIB)
        return _LIB


def _declare(L):
    P, S = ctypes.c_void_p, ctypes.c_size_t
    sigs = {
        "oracle_sha256": [P, S, P],
        "oracle_expand_message_xmd": [P, S, P, S, P, S],
        "oracle_expand_message_xof": [P, S, P, S, P, S],
        "oracle_shake256": [P, S, P, S],
        "oracle_set_suite": [ctypes.c_int],
        "oracle_hash_to_scalar": [P, S, P, S, P],
        "oracle_keygen": [P, S, P, S, P, S, P],
        "oracle_sk_to_pk": [P, P],
        "oracle_generators": [S, P, P],
        "oracle_hash_to_curve_g1": [P, S, P, S, P],
        "oracle_seeded_random_scalars": [P, S, P, S, S, P],
        "oracle_sign": [P, P, P, S, P, P, S, P, P, P],
        "oracle_verify": [P, P, S, P, S, P, P, S],
        "oracle_proof_gen": [P, P, S, P, S, P, S, P, P, S, P, S, P, S, P, S, P, S, P],
        "oracle_proof_verify": [P, P, S, P, S, P, S, P, P, S, P],
        "oracle_g1_msm": [P, P, S, P],
        "oracle_calculate_domain": [P, P, S, S, P],
        "oracle_g1_add": [P, P, P],
        "oracle_g1_decompress": [P, P],
        "oracle_g1_mul": [P, P, P],
        "oracle_g2_decompress": [P],
        "oracle_pairing_eq": [P, P, P, P],
        "oracle_fp_mul": [P, P, P],
        "oracle_fr_mul": [P, P, P],
        "oracle_fr_inv": [P, P],
    }
    for name, args in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int


def _suited(fn):
    """Adds a `suite` keyword (0 SHA-256, 1 SHAKE-256): the call runs with the
    oracle's per-thread ciphersuite set to it."""
    import functools

    @functools.wraps(fn)
    def run(*args, suite=SUITE_SHA256, **kw):
        L = lib()
        prev = L.oracle_set_suite(suite)
        if prev < 0:
            raise ValueError(f"unknown ciphersuite {suite}")
        prev_py = getattr(_TLS, "suite", SUITE_SHA256)
        _TLS.suite = suite
        try:
            return fn(*args, **kw)
        finally:
            _TLS.suite = prev_py
            L.oracle_set_suite(prev)
    return run


_TLS = threading.local()


def _buf(b: bytes):
    return ctypes.cast(ctypes.c_char_p(b), ctypes.c_void_p) if b else None


def _pack(msgs):
    data = b"".join(msgs)
    lens = (ctypes.c_size_t * max(1, len(msgs)))(*[len(m) for m in msgs])
    return data, lens


def sha256(msg: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    lib().oracle_sha256(_buf(msg), len(msg), out)
    return out.raw


def expand_message_xmd(msg: bytes, dst: bytes, n: int) -> bytes:
    out = ctypes.create_string_buffer(n)
    rc = lib().oracle_expand_message_xmd(_buf(msg), len(msg), _buf(dst), len(dst), out, n)
    if rc:
        raise ValueError("expand_message_xmd rejected its input")
    return out.raw


def expand_message_xof(msg: bytes, dst: bytes, n: int) -> bytes:
    out = ctypes.create_string_buffer(n)
    rc = lib().oracle_expand_message_xof(_buf(msg), len(msg), _buf(dst), len(dst), out, n)
    if rc:
        raise ValueError("expand_message_xof rejected its input")
    return out.raw


def shake256(msg: bytes, n: int) -> bytes:
    out = ctypes.create_string_buffer(n)
    lib().oracle_shake256(_buf(msg), len(msg), out, n)
    return out.raw


@_suited
def hash_to_scalar(msg: bytes, dst: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    if lib().oracle_hash_to_scalar(_buf(msg), len(msg), _buf(dst), len(dst), out):
        raise ValueError("hash_to_scalar rejected its input")
    return out.raw


@_suited
def keygen(key_material: bytes, key_info: bytes = b"", key_dst: bytes = None) -> bytes:
    out = ctypes.create_string_buffer(32)
    kd = key_dst if key_dst is not None else None
    rc = lib().oracle_keygen(_buf(key_material), len(key_material), _buf(key_info), len(key_info),
                             _buf(kd) if kd else None, len(kd) if kd else 0, out)
    if rc:
        raise ValueError("keygen rejected its input")
    return out.raw


def sk_to_pk(sk: bytes) -> bytes:
    out = ctypes.create_string_buffer(96)
    if lib().oracle_sk_to_pk(_buf(sk), out):
        raise ValueError("bad secret key")
    return out.raw


@_suited
def generators(count: int):
    out = ctypes.create_string_buffer(48 * count)
    p1 = ctypes.create_string_buffer(48)
    lib().oracle_generators(count, out, p1)
    return p1.raw, [out.raw[48 * i:48 * (i + 1)] for i in range(count)]


@_suited
def hash_to_curve_g1(msg: bytes, dst: bytes) -> bytes:
    out = ctypes.create_string_buffer(48)
    lib().oracle_hash_to_curve_g1(_buf(msg), len(msg), _buf(dst), len(dst), out)
    return out.raw


@_suited
def seeded_random_scalars(seed: bytes, dst: bytes, count: int):
    out = ctypes.create_string_buffer(32 * max(1, count))
    if lib().oracle_seeded_random_scalars(_buf(seed), len(seed), _buf(dst), len(dst), count, out):
        raise ValueError("seeded_random_scalars rejected its input")
    return [out.raw[32 * i:32 * (i + 1)] for i in range(count)]


@_suited
def sign(sk: bytes, pk: bytes, header: bytes, msgs):
    data, lens = _pack(msgs)
    sig = ctypes.create_string_buffer(80)
    b = ctypes.create_string_buffer(48)
    dom = ctypes.create_string_buffer(32)
    rc = lib().oracle_sign(_buf(sk), _buf(pk), _buf(header), len(header), _buf(data), lens,
                           len(msgs), sig, b, dom)
    if rc:
        return None
    return sig.raw, b.raw, dom.raw


@_suited
def verify(pk: bytes, sig: bytes, header: bytes, msgs) -> int:
    """0 valid, 2 invalid signature, 1 undecodable input."""
    data, lens = _pack(msgs)
    return lib().oracle_verify(_buf(pk), _buf(sig), len(sig), _buf(header), len(header),
                               _buf(data), lens, len(msgs))


@_suited
def proof_gen(pk, sig, header, ph, msgs, disclosed, seed=SEED_MOCKED_SCALAR, dst=None):
    if dst is None:  # the mocked-scalar DST of the call's suite
        dst = suite_dsts(_TLS.suite)[2]
    data, lens = _pack(msgs)
    idx = (ctypes.c_size_t * max(1, len(disclosed)))(*disclosed)
    cap = 512 + 48 * len(msgs) + 48 * len(disclosed) + 32 * len(msgs)
    out = ctypes.create_string_buffer(cap)
    n = ctypes.c_size_t(0)
    rc = lib().oracle_proof_gen(_buf(pk), _buf(sig), len(sig), _buf(header), len(header),
                                _buf(ph), len(ph), _buf(data), lens, len(msgs), idx,
                                len(disclosed), _buf(seed), len(seed), _buf(dst), len(dst),
                                out, cap, ctypes.byref(n))
    if rc:
        return None
    return out.raw[:n.value]


@_suited
def proof_verify(pk, proof, header, ph, disclosed_msgs, disclosed) -> int:
    """0 valid, 2 invalid proof, 1 undecodable public key."""
    data, lens = _pack(disclosed_msgs)
    idx = (ctypes.c_size_t * max(1, len(disclosed)))(*disclosed)
    return lib().oracle_proof_verify(_buf(pk), _buf(proof), len(proof), _buf(header),
                                     len(header), _buf(ph), len(ph), _buf(data), lens,
                                     len(disclosed_msgs), idx)


@_suited
def calculate_domain(pk: bytes, header: bytes, L: int) -> bytes:
    out = ctypes.create_string_buffer(32)
    if lib().oracle_calculate_domain(_buf(pk), _buf(header), len(header), L, out):
        raise ValueError("bad input")
    return out.raw


def g1_msm(points, scalars) -> bytes:
    out = ctypes.create_string_buffer(48)
    rc = lib().oracle_g1_msm(_buf(b"".join(points)), _buf(b"".join(scalars)), len(points), out)
    if rc:
        raise ValueError("bad MSM input")
    return out.raw


def g1_add(a: bytes, b: bytes) -> bytes:
    out = ctypes.create_string_buffer(48)
    if lib().oracle_g1_add(_buf(a), _buf(b), out):
        raise ValueError("bad point")
    return out.raw


def g1_mul(p: bytes, k: bytes) -> bytes:
    out = ctypes.create_string_buffer(48)
    if lib().oracle_g1_mul(_buf(p), _buf(k), out):
        raise ValueError("bad input")
    return out.raw


def g1_decompress(p: bytes):
    out = ctypes.create_string_buffer(96)
    if lib().oracle_g1_decompress(_buf(p), out):
        return None
    return out.raw


def g2_valid(p: bytes) -> bool:
    return lib().oracle_g2_decompress(_buf(p)) == 0


def pairing_eq(a, b, c, d) -> int:
    return lib().oracle_pairing_eq(_buf(a), _buf(b), _buf(c), _buf(d))


def fp_mul(a: bytes, b: bytes) -> bytes:
    out = ctypes.create_string_buffer(48)
    if lib().oracle_fp_mul(_buf(a), _buf(b), out):
        raise ValueError("non-canonical input")
    return out.raw


def fr_mul(a: bytes, b: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    if lib().oracle_fr_mul(_buf(a), _buf(b), out):
        raise ValueError("non-canonical input")
    return out.raw


def fr_inv(a: bytes) -> bytes:
    out = ctypes.create_string_buffer(32)
    if lib().oracle_fr_inv(_buf(a), out):
        raise ValueError("non-canonical input")
    return out.raw


P_MOD = int("1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab", 16)
R_MOD = int("73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001", 16)
