"""Python binding of libcubbs_bbs_cuda.so (the GB300 BBS drop-in) over ctypes.

The shared library exports the reference's C ABI v2 (include/cubbs_bbs_gpu_abi.h);
this module mirrors the ABI structs and offers batch helpers shaped like the
Rust loader's wrappers (crates/cubbs-bbs/src/gpu_runtime.rs:548-2196):
sign_batch / verify_batch / proof_gen_batch / proof_verify_batch and the
primitive MSM, hashing and pairing entry points.

There is no CPU path: loading fails loudly when the library is missing.
"""
import ctypes
import os
import pathlib
import threading

_HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib" / "libcubbs_bbs_cuda.so"
ABI_VERSION = 2

SUCCESS, ERR_INVALID_INPUT, ERR_INSUFFICIENT_OUTPUT, ERR_INTERNAL = 0, 1, 2, 3
ERR_NOALLOC_LIMIT = 4          # cubbs_bbs_gpu_g1_msm_noalloc_v2 only: too many terms
NOALLOC_MSM_MAX_TERMS = 4096   # term limit of cubbs_bbs_gpu_g1_msm_noalloc_v2
BACKEND_KIND_CUDA = 1
API_ID = b"BBS_BLS12381G1_XMD:SHA-256_SSWU_RO_H2G_HM2S_"
MAP_DST = API_ID + b"MAP_MSG_TO_SCALAR_AS_HASH_"
H2S_DST = API_ID + b"H2S_"
# ciphersuites (CUBBS_BBS_CIPHERSUITE_*): 0 BLS12-381-SHA-256, 1 BLS12-381-SHAKE-256
SUITE_SHA256, SUITE_SHAKE256 = 0, 1
API_ID_SHAKE256 = b"BBS_BLS12381G1_XOF:SHAKE-256_SSWU_RO_H2G_HM2S_"


class ByteSlice(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("len", ctypes.c_size_t)]


class ByteBuffer(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("capacity", ctypes.c_size_t), ("len", ctypes.c_size_t)]


class IndexSlice(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("len", ctypes.c_size_t)]


class Result(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("value", ctypes.c_uint8), ("bytes_written", ctypes.c_size_t)]


class BackendInfo(ctypes.Structure):
    _fields_ = [("backend_kind", ctypes.c_uint32), ("hardware_acceleration", ctypes.c_uint8)]


class SignItem(ctypes.Structure):
    _fields_ = [("secret_key", ByteSlice), ("public_key", ByteSlice), ("header", ByteSlice),
                ("messages", ctypes.c_void_p), ("message_count", ctypes.c_size_t), ("signature_out", ByteBuffer)]


class VerifyItem(ctypes.Structure):
    _fields_ = [("public_key", ByteSlice), ("signature", ByteSlice), ("header", ByteSlice),
                ("messages", ctypes.c_void_p), ("message_count", ctypes.c_size_t)]


class ProofGenItem(ctypes.Structure):
    _fields_ = [("public_key", ByteSlice), ("signature", ByteSlice), ("header", ByteSlice),
                ("presentation_header", ByteSlice), ("messages", ctypes.c_void_p),
                ("message_count", ctypes.c_size_t), ("disclosed_indexes", IndexSlice), ("proof_out", ByteBuffer)]


class ProofVerifyItem(ctypes.Structure):
    _fields_ = [("public_key", ByteSlice), ("proof", ByteSlice), ("header", ByteSlice),
                ("presentation_header", ByteSlice), ("disclosed_messages", ctypes.c_void_p),
                ("disclosed_count", ctypes.c_size_t), ("disclosed_indexes", IndexSlice),
                ("total_message_count", ctypes.c_size_t)]


class MessagesToScalarItem(ctypes.Structure):
    _fields_ = [("message", ByteSlice), ("dst", ByteSlice), ("scalar_out", ByteBuffer)]


class SignEFromResidentScalarsItem(ctypes.Structure):
    _fields_ = [("secret_key", ByteSlice), ("domain", ByteSlice), ("messages", ctypes.c_void_p),
                ("message_scalar_offset", ctypes.c_size_t), ("message_count", ctypes.c_size_t),
                ("message_scalars_out", ByteBuffer), ("scalar_out", ByteBuffer)]


class PrepareBItem(ctypes.Structure):
    _fields_ = [("public_key", ByteSlice), ("header", ByteSlice), ("message_scalars", ctypes.c_void_p),
                ("message_count", ctypes.c_size_t), ("b_out", ByteBuffer)]


class G1MsmItem(ctypes.Structure):
    _fields_ = [("points", ctypes.c_void_p), ("scalars", ctypes.c_void_p), ("term_count", ctypes.c_size_t),
                ("point_out", ByteBuffer)]


class G1MsmCommonPointsBatchItem(ctypes.Structure):
    _fields_ = [("points", ctypes.c_void_p), ("term_count", ctypes.c_size_t), ("scalar_rows", ctypes.c_void_p),
                ("scalar_rows_be", ctypes.c_void_p), ("scalar_row_stride", ctypes.c_size_t),
                ("output_count", ctypes.c_size_t), ("point_outs", ctypes.c_void_p)]


class G1MsmCommonPointsPlusVariableItem(ctypes.Structure):
    _fields_ = [("points", ctypes.c_void_p), ("term_count", ctypes.c_size_t), ("scalar_rows", ctypes.c_void_p),
                ("variable_points", ctypes.c_void_p), ("variable_scalars", ctypes.c_void_p),
                ("output_count", ctypes.c_size_t), ("point_outs", ctypes.c_void_p)]


class ProofVerifyMsmPairItem(ctypes.Structure):
    _fields_ = [("common_points", ctypes.c_void_p), ("common_term_count", ctypes.c_size_t),
                ("common_scalar_rows", ctypes.c_void_p), ("proof_points", ctypes.c_void_p),
                ("proof_scalars", ctypes.c_void_p), ("output_count", ctypes.c_size_t),
                ("t1_outs", ctypes.c_void_p), ("t2_outs", ctypes.c_void_p)]


class G1DualMsmSamePointsItem(ctypes.Structure):
    _fields_ = [("points", ctypes.c_void_p), ("lhs_scalars", ctypes.c_void_p), ("rhs_scalars", ctypes.c_void_p),
                ("term_count", ctypes.c_size_t), ("lhs_out", ByteBuffer), ("rhs_out", ByteBuffer)]


class G1DualMsmSamePointsLanesItem(ctypes.Structure):
    _fields_ = [("points", ctypes.c_void_p), ("lhs_scalars", ctypes.c_void_p), ("rhs_scalars", ctypes.c_void_p),
                ("term_count", ctypes.c_size_t), ("lane_count", ctypes.c_size_t), ("lhs_outs", ByteBuffer),
                ("rhs_outs", ByteBuffer)]


class G1AddItem(ctypes.Structure):
    _fields_ = [("lhs", ByteSlice), ("rhs", ByteSlice), ("point_out", ByteBuffer)]


class PairingEqItem(ctypes.Structure):
    _fields_ = [("lhs_g1", ByteSlice), ("lhs_g2", ByteSlice), ("rhs_g1", ByteSlice), ("rhs_g2", ByteSlice)]


class PairingEqScaledItem(ctypes.Structure):
    _fields_ = [("lhs_g1", ByteSlice), ("lhs_g2", ByteSlice), ("rhs_g1", ByteSlice), ("rhs_g2", ByteSlice),
                ("coefficient", ByteSlice)]


class ProofGenT2PrepareItem(ctypes.Structure):
    _fields_ = [("compressed_b", ByteSlice), ("signature_a", ByteSlice), ("scalars_be", ByteSlice * 7),
                ("seed", ByteSlice), ("d_out", ByteBuffer), ("abar_out", ByteBuffer), ("bbar_out", ByteBuffer),
                ("t1_out", ByteBuffer)]


class ProofValueBase(ctypes.Structure):
    _fields_ = [("bbs_signature", ByteSlice), ("bbs_header", ByteSlice), ("public_key", ByteSlice),
                ("hmac_key", ByteSlice), ("mandatory_pointers", ctypes.c_void_p),
                ("mandatory_pointer_count", ctypes.c_size_t)]


class ProofValueDerived(ctypes.Structure):
    _fields_ = [("bbs_proof", ByteSlice), ("label_keys", ctypes.c_void_p), ("label_values", ctypes.c_void_p),
                ("label_count", ctypes.c_size_t), ("mandatory_indexes", ctypes.c_void_p),
                ("mandatory_count", ctypes.c_size_t), ("selective_indexes", ctypes.c_void_p),
                ("selective_count", ctypes.c_size_t), ("presentation_header", ByteSlice)]


_LIB = None


def build():
    """Compile the CUDA library in-tree (sm_103a)."""
    from importlib import util
    spec = util.spec_from_file_location("_cubbs_build", _HERE / "build.py")
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def lib():
    """Load libcubbs_bbs_cuda.so; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run build() (no CPU fallback exists)")
        _LIB = ctypes.CDLL(str(LIB_PATH))
        U32, P, S = ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t
        special = {
            "cubbs_bbs_gpu_backend_info_v2": [U32, P],
            "cubbs_bbs_gpu_proof_gen_seeded_batch_v2": [U32, P, S, P, P],
            "cubbs_bbs_gpu_sign_e_from_resident_scalars_batch_v2": [U32, P, S, ByteSlice, ByteSlice, P],
            "cubbs_bbs_gpu_sha256_batch_for_test_v2": [U32, P, P, P, S, P],
            "cubbs_bbs_gpu_expand_xmd_sha256_48_batch_for_test_v2": [U32, P, P, P, S, P, S, P],
            "cubbs_bbs_gpu_hash_to_scalar_sha256_batch_for_test_v2": [U32, P, P, P, S, P, S, P],
            "cubbs_bbs_gpu_g1_msm_noalloc_v2": [U32, P, P, S, P, P],
            "cubbs_bbs_gpu_sign_batch_cs_v2": [U32, U32, P, S, P],
            "cubbs_bbs_gpu_verify_batch_cs_v2": [U32, U32, P, S, P],
            "cubbs_bbs_gpu_proof_gen_batch_cs_v2": [U32, U32, P, S, P],
            "cubbs_bbs_gpu_proof_gen_seeded_batch_cs_v2": [U32, U32, P, S, P, P],
            "cubbs_bbs_gpu_proof_verify_batch_cs_v2": [U32, U32, P, S, P],
            "cubbs_bbs_gpu_expand_xof_shake256_48_batch_for_test_v2": [U32, P, P, P, S, P, S, P],
            "cubbs_bbs_gpu_hash_to_scalar_shake256_batch_for_test_v2": [U32, P, P, P, S, P, S, P],
        }
        for name in _SYMBOLS:
            fn = getattr(_LIB, name)
            fn.restype = ctypes.c_int32
            fn.argtypes = special.get(name, [U32, P, S, P])
    return _LIB


_SYMBOLS = [
    "cubbs_bbs_gpu_backend_info_v2", "cubbs_bbs_gpu_sign_batch_v2", "cubbs_bbs_gpu_verify_batch_v2",
    "cubbs_bbs_gpu_proof_gen_batch_v2", "cubbs_bbs_gpu_proof_verify_batch_v2",
    "cubbs_bbs_gpu_proof_gen_seeded_batch_v2", "cubbs_bbs_gpu_messages_to_scalar_batch_v2",
    "cubbs_bbs_gpu_sign_e_from_resident_scalars_batch_v2", "cubbs_bbs_gpu_prepare_b_batch_v2",
    "cubbs_bbs_gpu_g1_msm_batch_v2", "cubbs_bbs_gpu_g1_msm_common_points_batch_v2",
    "cubbs_bbs_gpu_g1_msm_fused_common_points_batch_v2",
    "cubbs_bbs_gpu_g1_msm_common_points_plus_variable_batch_v2",
    "cubbs_bbs_gpu_proof_verify_msm_pair_batch_v2", "cubbs_bbs_gpu_g1_dual_msm_same_points_batch_v2",
    "cubbs_bbs_gpu_g1_dual_msm_same_points_lanes_batch_v2", "cubbs_bbs_gpu_g1_add_batch_v2",
    "cubbs_bbs_gpu_pairing_eq_batch_v2", "cubbs_bbs_gpu_pairing_eq_aggregate_v2",
    "cubbs_bbs_gpu_proof_gen_t2_prepare_batch_v2", "cubbs_bbs_gpu_sha256_batch_for_test_v2",
    "cubbs_bbs_gpu_expand_xmd_sha256_48_batch_for_test_v2",
    "cubbs_bbs_gpu_hash_to_scalar_sha256_batch_for_test_v2", "cubbs_bbs_gpu_g1_msm_noalloc_v2",
    "cubbs_bbs_gpu_sign_batch_cs_v2", "cubbs_bbs_gpu_verify_batch_cs_v2", "cubbs_bbs_gpu_proof_gen_batch_cs_v2",
    "cubbs_bbs_gpu_proof_gen_seeded_batch_cs_v2", "cubbs_bbs_gpu_proof_verify_batch_cs_v2",
    "cubbs_bbs_gpu_expand_xof_shake256_48_batch_for_test_v2",
    "cubbs_bbs_gpu_hash_to_scalar_shake256_batch_for_test_v2",
]


class _Keep:
    """Holds ctypes buffers alive for the duration of one call."""

    def __init__(self):
        self.refs = []

    def bytes(self, b: bytes):
        if not b:
            return ByteSlice(None, 0)
        buf = ctypes.create_string_buffer(bytes(b), len(b))
        self.refs.append(buf)
        return ByteSlice(ctypes.cast(buf, ctypes.c_void_p), len(b))

    def slices(self, items):
        arr = (ByteSlice * max(1, len(items)))(*[self.bytes(x) for x in items])
        self.refs.append(arr)
        return ctypes.cast(arr, ctypes.c_void_p)

    def out(self, cap: int):
        buf = ctypes.create_string_buffer(max(1, cap))
        self.refs.append(buf)
        return ByteBuffer(ctypes.cast(buf, ctypes.c_void_p), cap, 0), buf

    def index(self, idx):
        arr = (ctypes.c_size_t * max(1, len(idx)))(*idx)
        self.refs.append(arr)
        return IndexSlice(ctypes.cast(arr, ctypes.c_void_p), len(idx))


def _call(name, *args):
    conv = []
    for a in args:
        if isinstance(a, ctypes.Array):
            a = ctypes.cast(a, ctypes.c_void_p)
        elif isinstance(a, ctypes.Structure) and not isinstance(a, ByteSlice):
            a = ctypes.cast(ctypes.pointer(a), ctypes.c_void_p)
        conv.append(a)
    args = conv
    rc = getattr(lib(), name)(*args)
    if rc != SUCCESS:
        raise RuntimeError(f"{name} returned {rc}")


def backend_info():
    info = BackendInfo()
    _call("cubbs_bbs_gpu_backend_info_v2", ABI_VERSION, (info))
    return info.backend_kind, info.hardware_acceleration


def proof_capacity(message_count: int, disclosed_count: int) -> int:
    """Output capacity the Rust engine allocates (crates/cubbs-bbs/src/execution.rs:3726-3728)."""
    return 512 + message_count * 48 + disclosed_count * 48


def _op_call(name, suite, *args):
    """The *_batch_v2 entry for the SHA-256 suite, its *_batch_cs_v2 twin otherwise."""
    if suite == SUITE_SHA256:
        _call(name, ABI_VERSION, *args)
    else:
        _call(name.replace("_batch_v2", "_batch_cs_v2"), ABI_VERSION, suite, *args)


def sign_batch(reqs, suite=SUITE_SHA256):
    """reqs: list of (sk, pk, header, [messages]) -> list of (code, signature bytes)."""
    k = _Keep()
    items = (SignItem * len(reqs))()
    outs = []
    for i, (sk, pk, hdr, msgs) in enumerate(reqs):
        ob, buf = k.out(80)
        outs.append(buf)
        items[i] = SignItem(k.bytes(sk), k.bytes(pk), k.bytes(hdr), k.slices(msgs), len(msgs), ob)
    res = (Result * len(reqs))()
    _op_call("cubbs_bbs_gpu_sign_batch_v2", suite, items, len(reqs), res)
    return [(res[i].code, outs[i].raw[:items[i].signature_out.len]) for i in range(len(reqs))]


def verify_batch(reqs, suite=SUITE_SHA256):
    """reqs: list of (pk, signature, header, [messages]) -> list of (code, valid)."""
    k = _Keep()
    items = (VerifyItem * len(reqs))()
    for i, (pk, sig, hdr, msgs) in enumerate(reqs):
        items[i] = VerifyItem(k.bytes(pk), k.bytes(sig), k.bytes(hdr), k.slices(msgs), len(msgs))
    res = (Result * len(reqs))()
    _op_call("cubbs_bbs_gpu_verify_batch_v2", suite, items, len(reqs), res)
    return [(res[i].code, bool(res[i].value)) for i in range(len(reqs))]


def _proof_gen_items(k, reqs):
    items = (ProofGenItem * len(reqs))()
    outs = []
    for i, (pk, sig, hdr, ph, msgs, disclosed) in enumerate(reqs):
        ob, buf = k.out(proof_capacity(len(msgs), len(disclosed)))
        outs.append(buf)
        items[i] = ProofGenItem(k.bytes(pk), k.bytes(sig), k.bytes(hdr), k.bytes(ph), k.slices(msgs), len(msgs),
                                k.index(disclosed), ob)
    return items, outs


def proof_gen_batch(reqs, seeds=None, suite=SUITE_SHA256):
    """reqs: list of (pk, signature, header, ph, [messages], [disclosed]).  With seeds
    (one 32-byte seed per item) the blinding is deterministic; otherwise OS randomness."""
    k = _Keep()
    items, outs = _proof_gen_items(k, reqs)
    res = (Result * len(reqs))()
    if seeds is None:
        _op_call("cubbs_bbs_gpu_proof_gen_batch_v2", suite, items, len(reqs), res)
    else:
        sb = ctypes.create_string_buffer(b"".join(seeds), 32 * len(seeds))
        _op_call("cubbs_bbs_gpu_proof_gen_seeded_batch_v2", suite, items, len(reqs), sb, res)
    return [(res[i].code, outs[i].raw[:items[i].proof_out.len]) for i in range(len(reqs))]


def proof_verify_batch(reqs, suite=SUITE_SHA256):
    """reqs: list of (pk, proof, header, ph, [disclosed messages], [disclosed indexes], L)."""
    k = _Keep()
    items = (ProofVerifyItem * len(reqs))()
    for i, (pk, proof, hdr, ph, dmsgs, didx, L) in enumerate(reqs):
        items[i] = ProofVerifyItem(k.bytes(pk), k.bytes(proof), k.bytes(hdr), k.bytes(ph), k.slices(dmsgs),
                                   len(dmsgs), k.index(didx), L)
    res = (Result * len(reqs))()
    _op_call("cubbs_bbs_gpu_proof_verify_batch_v2", suite, items, len(reqs), res)
    return [(res[i].code, bool(res[i].value)) for i in range(len(reqs))]


def messages_to_scalar(msgs, dst=MAP_DST):
    k = _Keep()
    items = (MessagesToScalarItem * len(msgs))()
    outs = []
    for i, m in enumerate(msgs):
        ob, buf = k.out(32)
        outs.append(buf)
        items[i] = MessagesToScalarItem(k.bytes(m), k.bytes(dst), ob)
    res = (Result * len(msgs))()
    _call("cubbs_bbs_gpu_messages_to_scalar_batch_v2", ABI_VERSION, items, len(msgs), res)
    return [outs[i].raw[:32] for i in range(len(msgs))]


def _flat(msgs):
    data = b"".join(msgs)
    offs, cur = [], 0
    for m in msgs:
        offs.append(cur)
        cur += len(m)
    n = len(msgs)
    return (ctypes.create_string_buffer(data, max(1, len(data))), (ctypes.c_size_t * max(1, n))(*offs),
            (ctypes.c_size_t * max(1, n))(*[len(m) for m in msgs]))


def sha256_batch(msgs):
    d, o, l = _flat(msgs)
    out = ctypes.create_string_buffer(32 * max(1, len(msgs)))
    _call("cubbs_bbs_gpu_sha256_batch_for_test_v2", ABI_VERSION, d, o, l, ctypes.c_size_t(len(msgs)), out)
    return [out.raw[32 * i:32 * i + 32] for i in range(len(msgs))]


def expand_xmd48_batch(msgs, dst, suite=SUITE_SHA256):
    """48 bytes of the suite's expand_message (xmd over SHA-256 / xof over SHAKE-256) per message."""
    d, o, l = _flat(msgs)
    out = ctypes.create_string_buffer(48 * max(1, len(msgs)))
    name = ("cubbs_bbs_gpu_expand_xmd_sha256_48_batch_for_test_v2" if suite == SUITE_SHA256 else
            "cubbs_bbs_gpu_expand_xof_shake256_48_batch_for_test_v2")
    _call(name, ABI_VERSION, d, o, l, ctypes.c_size_t(len(msgs)), dst, ctypes.c_size_t(len(dst)), out)
    return [out.raw[48 * i:48 * i + 48] for i in range(len(msgs))]


def hash_to_scalar_batch(msgs, dst, suite=SUITE_SHA256):
    d, o, l = _flat(msgs)
    out = ctypes.create_string_buffer(32 * max(1, len(msgs)))
    name = ("cubbs_bbs_gpu_hash_to_scalar_sha256_batch_for_test_v2" if suite == SUITE_SHA256 else
            "cubbs_bbs_gpu_hash_to_scalar_shake256_batch_for_test_v2")
    _call(name, ABI_VERSION, d, o, l, ctypes.c_size_t(len(msgs)), dst, ctypes.c_size_t(len(dst)), out)
    return [out.raw[32 * i:32 * i + 32] for i in range(len(msgs))]


def g1_msm_batch(msms):
    """msms: list of ([points48], [scalars32]) -> list of (code, point48)."""
    k = _Keep()
    items = (G1MsmItem * len(msms))()
    outs = []
    for i, (pts, scs) in enumerate(msms):
        ob, buf = k.out(48)
        outs.append(buf)
        items[i] = G1MsmItem(k.slices(pts), k.slices(scs), len(pts), ob)
    res = (Result * len(msms))()
    _call("cubbs_bbs_gpu_g1_msm_batch_v2", ABI_VERSION, items, len(msms), res)
    return [(res[i].code, outs[i].raw[:48]) for i in range(len(msms))]


def g1_msm_noalloc(points, scalars):
    """One MSM through the allocation-free entry point (fixed scratch array in
    the library, at most NOALLOC_MSM_MAX_TERMS terms).  Returns (rc, code,
    point48): rc is the call's return value, code the per-item result code."""
    n = len(points)
    pb = ctypes.create_string_buffer(b"".join(points), max(1, 48 * n))
    sb = ctypes.create_string_buffer(b"".join(scalars), max(1, 32 * n))
    out = ctypes.create_string_buffer(48)
    res = Result()
    rc = lib().cubbs_bbs_gpu_g1_msm_noalloc_v2(ABI_VERSION, ctypes.cast(pb, ctypes.c_void_p),
                                               ctypes.cast(sb, ctypes.c_void_p), n,
                                               ctypes.cast(out, ctypes.c_void_p),
                                               ctypes.cast(ctypes.pointer(res), ctypes.c_void_p))
    return rc, res.code, out.raw[:48]

def g1_msm_common_points(points, rows, fused=False, packed_scale=None):
    """One group: common points, rows of scalars.  packed_scale: optional per-row
    scale factors, sent through the packed (K+1)*32 stride form."""
    k = _Keep()
    R = len(rows)
    outs = (ByteBuffer * max(1, R))()
    bufs = []
    for r in range(R):
        ob, buf = k.out(48)
        bufs.append(buf)
        outs[r] = ob
    item = G1MsmCommonPointsBatchItem()
    item.points = k.slices(points)
    item.term_count = len(points)
    if packed_scale is None:
        item.scalar_rows = k.slices([s for row in rows for s in row])
        item.scalar_rows_be = None
        item.scalar_row_stride = 0
    else:
        blob = b"".join(packed_scale[r] + b"".join(rows[r]) for r in range(R))
        b = ctypes.create_string_buffer(blob, max(1, len(blob)))
        k.refs.append(b)
        item.scalar_rows = None
        item.scalar_rows_be = ctypes.cast(b, ctypes.c_void_p)
        item.scalar_row_stride = (len(points) + 1) * 32
    item.output_count = R
    item.point_outs = ctypes.cast(outs, ctypes.c_void_p)
    res = (Result * max(1, R))()
    name = "cubbs_bbs_gpu_g1_msm_fused_common_points_batch_v2" if fused else "cubbs_bbs_gpu_g1_msm_common_points_batch_v2"
    _call(name, ABI_VERSION, (item), 1, res)
    return [(res[r].code, res[r].value, bufs[r].raw[:48]) for r in range(R)]


def prepared_common_points_call(points, rows):
    """Builds one common-points group (packed big-endian scalar rows) once and
    returns call() -> [(code, route, point48)] making one synchronous
    cubbs_bbs_gpu_g1_msm_common_points_batch_v2 call on it."""
    k = _Keep()
    R = len(rows)
    outs = (ByteBuffer * max(1, R))()
    bufs = []
    for r in range(R):
        ob, buf = k.out(48)
        bufs.append(buf)
        outs[r] = ob
    blob = b"".join(b"".join(row) for row in rows)
    b = ctypes.create_string_buffer(blob, max(1, len(blob)))
    k.refs.append(b)
    item = G1MsmCommonPointsBatchItem()
    item.points = k.slices(points)
    item.term_count = len(points)
    item.scalar_rows = None
    item.scalar_rows_be = ctypes.cast(b, ctypes.c_void_p)
    item.scalar_row_stride = len(points) * 32
    item.output_count = R
    item.point_outs = ctypes.cast(outs, ctypes.c_void_p)
    res = (Result * max(1, R))()
    fn = lib().cubbs_bbs_gpu_g1_msm_common_points_batch_v2
    ip, rp = ctypes.cast(ctypes.pointer(item), ctypes.c_void_p), ctypes.cast(res, ctypes.c_void_p)

    def call():
        rc = fn(ABI_VERSION, ip, 1, rp)
        if rc:
            raise RuntimeError(f"common points call returned {rc}")
        _ = k
        return [(res[r].code, res[r].value, bufs[r].raw[:48]) for r in range(R)]
    return call


def msm_uneven_bench(n_msms=16384, k_min=2, k_max=257, seed=4, tune=True, warmup=3, steps=5):
    """Uneven variable-base MSM benchmark (points u*P1 and scalars generated on the
    device from `seed`).  Returns dict(ms=[per replay], decode_ms, chunk=[per size
    class], window=[per size class], checked, mismatch)."""
    ms = (ctypes.c_float * steps)()
    dec = ctypes.c_float(0)
    tun = (ctypes.c_uint32 * 12)()
    chk, mm = ctypes.c_uint32(0), ctypes.c_uint32(0)
    fn = lib().cubbs_bbs_gpu_msm_uneven_bench_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                   ctypes.c_int32, ctypes.c_int32, ctypes.c_int32] + [ctypes.c_void_p] * 5
    rc = fn(ABI_VERSION, n_msms, k_min, k_max, seed, 1 if tune else 0, warmup, steps, ctypes.cast(ms, ctypes.c_void_p),
            ctypes.cast(ctypes.pointer(dec), ctypes.c_void_p), ctypes.cast(tun, ctypes.c_void_p),
            ctypes.cast(ctypes.pointer(chk), ctypes.c_void_p), ctypes.cast(ctypes.pointer(mm), ctypes.c_void_p))
    if rc:
        raise RuntimeError(f"msm_uneven_bench returned {rc}")
    return {"ms": list(ms), "decode_ms": dec.value, "chunk": list(tun[:4]), "window": list(tun[4:8]),
            "mode": list(tun[8:]),
            "checked": chk.value, "mismatch": mm.value}


def msm_tuning(chunk=None, window=None, mode=None):
    """Uneven-MSM engine settings per size class (K <= 8, <= 32, <= 96, larger):
    with chunk, window and mode (4 values each; mode 0 thread, 1 warp; mode
    defaults to thread) they replace the process's settings.  Returns the
    (chunk, window, mode) lists in force."""
    fn = lib().cubbs_bbs_gpu_msm_tuning_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p] * 6
    if chunk is not None and mode is None:
        mode = [0] * 4
    arrs = [(ctypes.c_uint32 * 4)(*v) if v is not None else None for v in (chunk, window, mode)]
    outs = [(ctypes.c_uint32 * 4)() for _ in range(3)]
    args = [ctypes.cast(a, ctypes.c_void_p) if a is not None else None for a in arrs]
    args += [ctypes.cast(o, ctypes.c_void_p) for o in outs]
    rc = fn(*args)
    if rc:
        raise ValueError(f"msm_tuning returned {rc}")
    return tuple(list(o) for o in outs)


def sm_partition():
    """(small, rest) SM counts of the ProofVerify SM partition: the aggregated
    pairing check runs alone on `small` SMs, everything else on `rest`; (0, 0)
    when the partition is off (driver without green contexts, or
    CUBBS_BBS_SM_PARTITION=0), with the reason as a third value (0 when on)."""
    a, b, st = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
    fn = lib().cubbs_bbs_gpu_sm_partition_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    if fn(*(ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in (a, b, st))):
        raise RuntimeError("sm_partition failed")
    return a.value, b.value, st.value


def sm_partition_var():
    """(SMs, status) of the third ProofVerify partition, split off `rest`: the
    point decode and the variable-base terms run there alone (0 SMs when off;
    status 0 when on, else why it is off)."""
    v, st = ctypes.c_int32(0), ctypes.c_int32(0)
    fn = lib().cubbs_bbs_gpu_sm_partition_var_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    if fn(*(ctypes.cast(ctypes.pointer(x), ctypes.c_void_p) for x in (v, st))):
        raise RuntimeError("sm_partition_var failed")
    return v.value, st.value


def table_window():
    """Window width of the resident fixed-base table (0 before it is built)."""
    w = ctypes.c_int32(0)
    fn = lib().cubbs_bbs_gpu_table_window_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p]
    if fn(ctypes.cast(ctypes.pointer(w), ctypes.c_void_p)):
        raise RuntimeError("table_window failed")
    return w.value


def fixed_msm_autotune(scalars_be, rows, terms, w_lo=4, w_hi=20, steps=3, with_mismatches=False):
    """Times the fixed-base MSM kernel over rows x terms scalars (bases: the first
    `terms` resident generators) for table window widths w_lo..w_hi, after
    checking each width's first 64 rows against a table-free recomputation; the
    fastest agreeing width stays in use.  Returns ([ms per width; -1 for a width
    that disagreed], best width) and, with with_mismatches, the mismatch count."""
    nw = w_hi - w_lo + 1
    ms = (ctypes.c_float * nw)()
    best = ctypes.c_int32(0)
    bad = ctypes.c_int32(0)
    sb = ctypes.create_string_buffer(scalars_be, len(scalars_be))
    fn = lib().cubbs_bbs_gpu_fixed_msm_autotune_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    rc = fn(ABI_VERSION, ctypes.cast(sb, ctypes.c_void_p), rows, terms, w_lo, w_hi, steps,
            ctypes.cast(ms, ctypes.c_void_p), ctypes.cast(ctypes.pointer(best), ctypes.c_void_p),
            ctypes.cast(ctypes.pointer(bad), ctypes.c_void_p))
    if rc:
        raise RuntimeError(f"fixed_msm_autotune returned {rc} ({bad.value} widths disagreed)")
    if with_mismatches:
        return list(ms), best.value, bad.value
    return list(ms), best.value


def g1_msm_common_points_plus_variable(points, rows, var_points, var_scalars):
    k = _Keep()
    R = len(rows)
    outs = (ByteBuffer * max(1, R))()
    bufs = []
    for r in range(R):
        ob, buf = k.out(48)
        bufs.append(buf)
        outs[r] = ob
    item = G1MsmCommonPointsPlusVariableItem(k.slices(points), len(points), k.slices([s for row in rows for s in row]),
                                             k.slices(var_points), k.slices(var_scalars), R,
                                             ctypes.cast(outs, ctypes.c_void_p))
    res = (Result * max(1, R))()
    _call("cubbs_bbs_gpu_g1_msm_common_points_plus_variable_batch_v2", ABI_VERSION, (item), 1, res)
    return [(res[r].code, bufs[r].raw[:48]) for r in range(R)]


def proof_verify_msm_pair(points, rows, proof_points, proof_scalars):
    """proof_points rows [Bbar, Abar, D]; proof_scalars rows [c, e^, r1^, r3^]."""
    k = _Keep()
    R = len(rows)
    t1 = (ByteBuffer * max(1, R))()
    t2 = (ByteBuffer * max(1, R))()
    b1, b2 = [], []
    for r in range(R):
        o1, x1 = k.out(48)
        o2, x2 = k.out(48)
        t1[r], t2[r] = o1, o2
        b1.append(x1)
        b2.append(x2)
    item = ProofVerifyMsmPairItem(k.slices(points), len(points), k.slices([s for row in rows for s in row]),
                                  k.slices([p for row in proof_points for p in row]),
                                  k.slices([s for row in proof_scalars for s in row]), R,
                                  ctypes.cast(t1, ctypes.c_void_p), ctypes.cast(t2, ctypes.c_void_p))
    res = (Result * max(1, R))()
    _call("cubbs_bbs_gpu_proof_verify_msm_pair_batch_v2", ABI_VERSION, (item), 1, res)
    return [(res[r].code, b1[r].raw[:48], b2[r].raw[:48]) for r in range(R)]


def g1_dual_msm_same_points(points, lhs, rhs, lanes=None):
    k = _Keep()
    if lanes is None:
        o1, x1 = k.out(48)
        o2, x2 = k.out(48)
        item = G1DualMsmSamePointsItem(k.slices(points), k.slices(lhs), k.slices(rhs), len(points), o1, o2)
        res = Result()
        _call("cubbs_bbs_gpu_g1_dual_msm_same_points_batch_v2", ABI_VERSION, (item), 1, (res))
        return res.code, x1.raw[:48], x2.raw[:48]
    o1, x1 = k.out(48 * lanes)
    o2, x2 = k.out(48 * lanes)
    item = G1DualMsmSamePointsLanesItem(k.slices(points), k.slices(lhs), k.slices(rhs), len(points), lanes, o1, o2)
    res = Result()
    _call("cubbs_bbs_gpu_g1_dual_msm_same_points_lanes_batch_v2", ABI_VERSION, (item), 1,
          (res))
    return res.code, [x1.raw[48 * j:48 * j + 48] for j in range(lanes)], [x2.raw[48 * j:48 * j + 48] for j in range(lanes)]


def g1_add_batch(pairs):
    k = _Keep()
    items = (G1AddItem * len(pairs))()
    bufs = []
    for i, (a, b) in enumerate(pairs):
        ob, buf = k.out(48)
        bufs.append(buf)
        items[i] = G1AddItem(k.bytes(a), k.bytes(b), ob)
    res = (Result * len(pairs))()
    _call("cubbs_bbs_gpu_g1_add_batch_v2", ABI_VERSION, items, len(pairs), res)
    return [(res[i].code, bufs[i].raw[:48]) for i in range(len(pairs))]


def prepare_b_batch(reqs):
    """reqs: list of (pk, header64, [message scalars])."""
    k = _Keep()
    items = (PrepareBItem * len(reqs))()
    bufs = []
    for i, (pk, hdr, scs) in enumerate(reqs):
        ob, buf = k.out(48)
        bufs.append(buf)
        items[i] = PrepareBItem(k.bytes(pk), k.bytes(hdr), k.slices(scs), len(scs), ob)
    res = (Result * len(reqs))()
    _call("cubbs_bbs_gpu_prepare_b_batch_v2", ABI_VERSION, items, len(reqs), res)
    return [(res[i].code, bufs[i].raw[:48]) for i in range(len(reqs))]


def proof_gen_t2_prepare(reqs):
    """reqs: list of (B48, A48, [7 scalars]) -> list of (code, d, abar, bbar, t1)."""
    k = _Keep()
    items = (ProofGenT2PrepareItem * len(reqs))()
    bufs = []
    for i, (b, a, scs) in enumerate(reqs):
        it = ProofGenT2PrepareItem()
        it.compressed_b = k.bytes(b)
        it.signature_a = k.bytes(a)
        for s in range(7):
            it.scalars_be[s] = k.bytes(scs[s])
        it.seed = k.bytes(bytes(32))
        outs = []
        for f in ("d_out", "abar_out", "bbar_out", "t1_out"):
            ob, buf = k.out(48)
            setattr(it, f, ob)
            outs.append(buf)
        bufs.append(outs)
        items[i] = it
    res = (Result * len(reqs))()
    _call("cubbs_bbs_gpu_proof_gen_t2_prepare_batch_v2", ABI_VERSION, items, len(reqs), res)
    return [(res[i].code, *[b.raw[:48] for b in bufs[i]]) for i in range(len(reqs))]


def pairing_eq_batch(reqs):
    """reqs: list of (a48, b96, c48, d96): value = e(a, b) == e(c, d)."""
    k = _Keep()
    items = (PairingEqItem * len(reqs))()
    for i, (a, b, c, d) in enumerate(reqs):
        items[i] = PairingEqItem(k.bytes(a), k.bytes(b), k.bytes(c), k.bytes(d))
    res = (Result * len(reqs))()
    _call("cubbs_bbs_gpu_pairing_eq_batch_v2", ABI_VERSION, items, len(reqs), res)
    return [(res[i].code, bool(res[i].value)) for i in range(len(reqs))]


def g1_msm_pairing_batch(msms, pairs):
    """Uneven MSMs ([points48], [scalars32]) and pairing checks (a48, b96, c48,
    d96) in one persistent launch -> ([(code, point48)], [(code, e(a,b) == e(c,d))])."""
    k = _Keep()
    mitems = (G1MsmItem * max(1, len(msms)))()
    outs = []
    for i, (pts, scs) in enumerate(msms):
        ob, buf = k.out(48)
        outs.append(buf)
        mitems[i] = G1MsmItem(k.slices(pts), k.slices(scs), len(pts), ob)
    pitems = (PairingEqItem * max(1, len(pairs)))()
    for i, (a, b, c, d) in enumerate(pairs):
        pitems[i] = PairingEqItem(k.bytes(a), k.bytes(b), k.bytes(c), k.bytes(d))
    mres = (Result * max(1, len(msms)))()
    pres = (Result * max(1, len(pairs)))()
    fn = lib().cubbs_bbs_gpu_g1_msm_pairing_batch_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_void_p]
    rc = fn(ABI_VERSION, ctypes.cast(mitems, ctypes.c_void_p), len(msms), ctypes.cast(pitems, ctypes.c_void_p),
            len(pairs), ctypes.cast(mres, ctypes.c_void_p), ctypes.cast(pres, ctypes.c_void_p))
    if rc:
        raise RuntimeError(f"g1_msm_pairing_batch returned {rc}")
    return ([(mres[i].code, outs[i].raw[:48]) for i in range(len(msms))],
            [(pres[i].code, bool(pres[i].value)) for i in range(len(pairs))])


def pairing_eq_aggregate(reqs):
    """reqs: list of (a48, b96, c48, d96, coef32) -> (code, value)."""
    k = _Keep()
    items = (PairingEqScaledItem * max(1, len(reqs)))()
    for i, (a, b, c, d, co) in enumerate(reqs):
        items[i] = PairingEqScaledItem(k.bytes(a), k.bytes(b), k.bytes(c), k.bytes(d), k.bytes(co))
    res = Result()
    _call("cubbs_bbs_gpu_pairing_eq_aggregate_v2", ABI_VERSION, items, len(reqs), (res))
    return res.code, bool(res.value)


def fp_op_for_test(op, a_list, b_list):
    """Device Fp op (0 mul, 1 inverse, 2 sqrt, 3 variable-time inverse, 4 CIOS mul) on
    48-byte BE canonical inputs."""
    n = len(a_list)
    a = ctypes.create_string_buffer(b"".join(a_list), max(1, 48 * n))
    b = ctypes.create_string_buffer(b"".join(b_list), max(1, 48 * n))
    out = ctypes.create_string_buffer(max(1, 48 * n))
    st = (ctypes.c_int32 * max(1, n))()
    fn = lib().cubbs_bbs_gpu_fp_op_for_test_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_void_p]
    rc = fn(ABI_VERSION, op, ctypes.cast(a, ctypes.c_void_p), ctypes.cast(b, ctypes.c_void_p), n,
            ctypes.cast(out, ctypes.c_void_p), ctypes.cast(st, ctypes.c_void_p))
    if rc:
        raise RuntimeError(f"fp_op_for_test returned {rc}")
    return [(st[i], out.raw[48 * i:48 * i + 48]) for i in range(n)]


def g1_op_for_test(points, scalars):
    """Device decode (status 0 ok, 1 identity, 2 rejected) -> (status, x||y, k*P compressed)."""
    n = len(points)
    p = ctypes.create_string_buffer(b"".join(points), max(1, 48 * n))
    k = ctypes.create_string_buffer(b"".join(scalars), max(1, 32 * n))
    xy = ctypes.create_string_buffer(max(1, 96 * n))
    kp = ctypes.create_string_buffer(max(1, 48 * 77 * n))
    st = (ctypes.c_int32 * max(1, n))()
    fn = lib().cubbs_bbs_gpu_g1_op_for_test_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32] + [ctypes.c_void_p] * 2 + [ctypes.c_size_t] + [ctypes.c_void_p] * 3
    rc = fn(ABI_VERSION, ctypes.cast(p, ctypes.c_void_p), ctypes.cast(k, ctypes.c_void_p), n,
            ctypes.cast(xy, ctypes.c_void_p), ctypes.cast(kp, ctypes.c_void_p), ctypes.cast(st, ctypes.c_void_p))
    if rc:
        raise RuntimeError(f"g1_op_for_test returned {rc}")
    diag = [[kp.raw[48 * (n + 12 * i + j):48 * (n + 12 * i + j + 1)] for j in range(12)] for i in range(n)]
    chain = [[kp.raw[48 * (13 * n + 64 * i + j):48 * (13 * n + 64 * i + j + 1)] for j in range(64)] for i in range(n)]
    return [(st[i], xy.raw[96 * i:96 * i + 96], kp.raw[48 * i:48 * i + 48], diag[i], chain[i]) for i in range(n)]


def g1_subgroup_for_test(points):
    """Unchecked device decode plus the separate subgroup kernel -> [(decode status, outside G1)]."""
    n = len(points)
    p = ctypes.create_string_buffer(b"".join(points), max(1, 48 * n))
    st = (ctypes.c_int32 * max(1, n))()
    out = (ctypes.c_int32 * max(1, n))()
    fn = lib().cubbs_bbs_gpu_g1_subgroup_for_test_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    rc = fn(ABI_VERSION, ctypes.cast(p, ctypes.c_void_p), n, ctypes.cast(st, ctypes.c_void_p),
            ctypes.cast(out, ctypes.c_void_p))
    if rc:
        raise RuntimeError(f"g1_subgroup_for_test returned {rc}")
    return [(st[i], out[i]) for i in range(n)]


# --------------------------------------------------------------------------- benchmark helpers
OP_SIGN, OP_VERIFY, OP_PROOF_GEN, OP_PROOF_VERIFY = 0, 1, 2, 3


def _op_items(op, reqs, k):
    if op == OP_SIGN:
        items = (SignItem * len(reqs))()
        for i, (sk, pk, hdr, msgs) in enumerate(reqs):
            ob, _ = k.out(80)
            items[i] = SignItem(k.bytes(sk), k.bytes(pk), k.bytes(hdr), k.slices(msgs), len(msgs), ob)
        return items
    if op == OP_VERIFY:
        items = (VerifyItem * len(reqs))()
        for i, (pk, sig, hdr, msgs) in enumerate(reqs):
            items[i] = VerifyItem(k.bytes(pk), k.bytes(sig), k.bytes(hdr), k.slices(msgs), len(msgs))
        return items
    if op == OP_PROOF_GEN:
        items, _ = _proof_gen_items(k, reqs)
        return items
    items = (ProofVerifyItem * len(reqs))()
    for i, (pk, proof, hdr, ph, dmsgs, didx, L) in enumerate(reqs):
        items[i] = ProofVerifyItem(k.bytes(pk), k.bytes(proof), k.bytes(hdr), k.bytes(ph), k.slices(dmsgs),
                                   len(dmsgs), k.index(didx), L)
    return items


class ServeConfig(ctypes.Structure):
    _fields_ = [("max_inflight", ctypes.c_uint32), ("max_batch_items", ctypes.c_uint32),
                ("hbm_budget_bytes", ctypes.c_uint64)]


SERVE_QUEUE, SERVE_PLAIN = 0, 1


def serve_replay(pool, schedule, mode=SERVE_QUEUE, max_inflight=0, max_batch_items=0, hbm_budget_bytes=0,
                 plain_batch=256, plain_timeout_us=2000):
    """Replays single requests through the serving queue (mode 0) or through plain
    fixed-size batches (mode 1).  pool: list of (op, req, seed or None), req shaped
    as for the batch helpers (OP_SIGN ... OP_PROOF_VERIFY); schedule: list of
    (pool index, arrival offset in ns), offsets non-decreasing.  A pool entry may be
    scheduled more than once (its output buffer is then shared).  Returns
    (results, latencies_ns, wall_s), results[i] = (code, value, output bytes or None)."""
    k = _Keep()
    P, n = len(pool), len(schedule)
    pool_ptr = [0] * P
    outs = [None] * P
    arrays = []
    for op in (OP_SIGN, OP_VERIFY, OP_PROOF_GEN, OP_PROOF_VERIFY):
        idxs = [i for i, (o, _, _) in enumerate(pool) if o == op]
        if not idxs:
            continue
        reqs = [pool[i][1] for i in idxs]
        if op == OP_SIGN:
            items = (SignItem * len(reqs))()
            bufs = []
            for j, (sk, pk, hdr, msgs) in enumerate(reqs):
                ob, buf = k.out(80)
                bufs.append(buf)
                items[j] = SignItem(k.bytes(sk), k.bytes(pk), k.bytes(hdr), k.slices(msgs), len(msgs), ob)
        elif op == OP_PROOF_GEN:
            items, bufs = _proof_gen_items(k, reqs)
        else:
            items, bufs = _op_items(op, reqs, k), None
        arrays.append(items)
        for j, i in enumerate(idxs):
            pool_ptr[i] = ctypes.addressof(items[j])
            if bufs is not None:
                outs[i] = (items, j, bufs[j])
    ptrs = (ctypes.c_void_p * max(1, n))(*[pool_ptr[i] for i, _ in schedule])
    ops = (ctypes.c_int32 * max(1, n))(*[pool[i][0] for i, _ in schedule])
    seeds = ctypes.create_string_buffer(32 * max(1, n))
    has_seed = False
    for s, (i, _) in enumerate(schedule):
        if pool[i][2] is not None:
            ctypes.memmove(ctypes.addressof(seeds) + 32 * s, pool[i][2], 32)
            has_seed = True
    arr = (ctypes.c_uint64 * max(1, n))(*[a for _, a in schedule])
    lat = (ctypes.c_uint64 * max(1, n))()
    res = (Result * max(1, n))()
    wall = ctypes.c_double(0)
    cfg = ServeConfig(max_inflight, max_batch_items, hbm_budget_bytes)
    fn = lib().cubbs_bbs_gpu_serve_replay
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    rc = fn(ABI_VERSION, mode, ctypes.cast(ctypes.pointer(cfg), ctypes.c_void_p), ctypes.cast(ops, ctypes.c_void_p),
            ctypes.cast(ptrs, ctypes.c_void_p), ctypes.cast(seeds, ctypes.c_void_p) if has_seed else None,
            ctypes.cast(arr, ctypes.c_void_p), n, plain_batch, plain_timeout_us, ctypes.cast(lat, ctypes.c_void_p),
            ctypes.cast(res, ctypes.c_void_p), ctypes.cast(ctypes.pointer(wall), ctypes.c_void_p))
    if rc:
        raise RuntimeError(f"serve_replay returned {rc}")
    results = []
    for s, (i, _) in enumerate(schedule):
        out = None
        if outs[i] is not None:
            items, j, buf = outs[i]
            ln = items[j].signature_out.len if pool[i][0] == OP_SIGN else items[j].proof_out.len
            out = buf.raw[:ln]
        results.append((res[s].code, res[s].value, out))
    del arrays
    return results, [lat[s] for s in range(n)], wall.value


class ServeQueueConfig(ctypes.Structure):
    _fields_ = [("max_batch_items", ctypes.c_uint32), ("max_inflight", ctypes.c_uint32),
                ("coalesce_us", ctypes.c_uint32), ("queue_capacity", ctypes.c_uint32)]


class ServeSnapshot(ctypes.Structure):
    _fields_ = [("queued", ctypes.c_uint64), ("dispatches", ctypes.c_uint64), ("dispatched_items", ctypes.c_uint64),
                ("max_observed_batch", ctypes.c_uint64), ("last_batch_size", ctypes.c_uint64),
                ("inflight_batches", ctypes.c_uint64), ("total_queue_wait_ms", ctypes.c_double),
                ("average_queue_wait_ms", ctypes.c_double)]


SERVE_MAX_QUEUES = 8


def serve_queue(op, suite=0):
    """Device serving queue of operation op (OP_*) under a ciphersuite (SUITE_*)."""
    return op + 4 * suite

_SERVE_DONE = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(Result))
_SERVE_PROCESSOR = ctypes.CFUNCTYPE(ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                    ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t, ctypes.POINTER(Result))


class ServeReceiver:
    """The reply to one enqueued request (BatchReceiver, batcher.rs:107-115)."""

    def __init__(self, callback=None):
        self._event = threading.Event()
        self._value = None
        self._callback = callback
        self.ticket = 0

    def _set(self, value):
        self._value = value
        self._event.set()
        if self._callback is not None:
            self._callback(value)

    def done(self):
        return self._event.is_set()

    def _attach(self, keep, items, buf, op):
        self._keep, self._items, self._buf, self._op = keep, items, buf, op

    def output(self):
        """Signature or proof bytes of a device Sign / ProofGen request."""
        buf = getattr(self, "_buf", None)
        if buf is None or not self._event.is_set():
            return None
        item = self._items[0]
        n = item.signature_out.len if self._op == OP_SIGN else item.proof_out.len
        return buf.raw[:n]

    def receive(self, timeout=None):
        """(code, value, bytes_written) of the request; raises TimeoutError."""
        if not self._event.wait(timeout):
            raise TimeoutError("serving queue did not reply in time")
        return self._value


class ServeQueue:
    """Client of the native serving queue in the shape of the reference W3C
    service's BatchQueue (crates/cubbs-w3c-service/src/batcher.rs:118-221):
    per-queue batcher settings (configure / configure_batcher / config),
    enqueue -> ServeReceiver, submit, snapshot.

    processor=None: the queues are the four BBS operations on the device (queue
    = OP_*, items are ABI item structs that stay alive until their reply).
    Otherwise processor(queue, items) -> [(code, value, bytes_written)] is
    called on a dispatch thread with a batch of the caller's objects, the
    batcher's generic processor; it raising fails the batch with ERR_INTERNAL."""

    def __init__(self, processor=None, max_inflight=0, max_batch_items=0, hbm_budget_bytes=0):
        self._lib = lib()
        self._handle = ctypes.c_void_p()
        self._mu = threading.Lock()
        self._pending = {}
        self._objects = {}
        self._next = 1
        self._processor = processor
        self._done_cb = _SERVE_DONE(self._on_done)
        self._submit = self._lib.cubbs_bbs_gpu_serve_submit_notify
        self._submit.restype = ctypes.c_int32
        self._submit.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_char_p, _SERVE_DONE,
                                 ctypes.c_void_p, ctypes.c_void_p]
        cfg = ServeConfig(max_inflight, max_batch_items, hbm_budget_bytes)
        if processor is None:
            self._proc_cb = None
            rc = self._lib.cubbs_bbs_gpu_serve_create(ABI_VERSION, ctypes.byref(cfg), ctypes.byref(self._handle))
        else:
            self._proc_cb = _SERVE_PROCESSOR(self._on_batch)
            fn = self._lib.cubbs_bbs_gpu_serve_create_with_processor
            fn.argtypes = [ctypes.c_uint32, ctypes.c_void_p, _SERVE_PROCESSOR, ctypes.c_void_p, ctypes.c_void_p]
            rc = fn(ABI_VERSION, ctypes.addressof(cfg), self._proc_cb, None, ctypes.addressof(self._handle))
        if rc:
            raise RuntimeError(f"serve_create returned {rc}")

    def _on_batch(self, _ctx, queue, items, n, results):
        try:
            with self._mu:
                objs = [self._objects[items[i]][0] for i in range(n)]
            outs = list(self._processor(queue, objs))
            for i in range(n):
                code, value, written = outs[i] if i < len(outs) else (ERR_INTERNAL, 0, 0)
                results[i].code, results[i].value, results[i].bytes_written = code, value, written
            return SUCCESS
        except Exception:  # noqa: BLE001 - a failing processor fails its batch
            return ERR_INTERNAL

    def _on_done(self, ctx, _ticket, result):
        r = result.contents
        with self._mu:
            rec = self._pending.pop(ctx)
            self._objects.pop(ctx, None)
        rec._set((r.code, r.value, r.bytes_written))

    def configure(self, queue, max_batch_items=0, max_inflight=0, coalesce_us=0, queue_capacity=0):
        """Sets one queue's settings; returns those in force (config())."""
        cfg = ServeQueueConfig(max_batch_items, max_inflight, coalesce_us, queue_capacity)
        eff = ServeQueueConfig()
        rc = self._lib.cubbs_bbs_gpu_serve_configure_queue(self._handle, queue, ctypes.byref(cfg), ctypes.byref(eff))
        if rc:
            raise ValueError(f"serve_configure_queue returned {rc}")
        return {f: getattr(eff, f) for f, _ in ServeQueueConfig._fields_}

    def configure_batcher(self, queue, interval_ms, max_batch_size, queue_capacity, pipelines):
        """configure() from the reference's BatcherConfig fields (batcher.rs:21-27)."""
        return self.configure(queue, max_batch_size, pipelines, interval_ms * 1000, queue_capacity)

    def config(self, queue):
        eff = ServeQueueConfig()
        rc = self._lib.cubbs_bbs_gpu_serve_configure_queue(self._handle, queue, None, ctypes.byref(eff))
        if rc:
            raise ValueError(f"serve_configure_queue returned {rc}")
        return {f: getattr(eff, f) for f, _ in ServeQueueConfig._fields_}

    def enqueue(self, queue, item, seed=None, callback=None):
        """Queues one request and returns its ServeReceiver; waits while the
        queue is at its capacity (BatchQueue::enqueue, batcher.rs:171-190).
        callback(reply), if given, runs on the dispatch thread when the reply
        arrives (for event-loop clients); it may enqueue again."""
        rec = ServeReceiver(callback)
        with self._mu:
            key = self._next
            self._next += 1
            self._pending[key] = rec
            if self._processor is not None:
                self._objects[key] = (item,)
        ptr = key if self._processor is not None else ctypes.addressof(item)
        ticket = ctypes.c_uint64()
        rc = self._submit(self._handle, queue, ptr, seed, self._done_cb, key, ctypes.addressof(ticket))
        if rc:
            with self._mu:
                self._pending.pop(key, None)
                self._objects.pop(key, None)
            raise ValueError(f"serve_submit_notify returned {rc}")
        rec.ticket = ticket.value
        return rec

    def submit(self, queue, item, seed=None, timeout=None):
        return self.enqueue(queue, item, seed).receive(timeout)

    def enqueue_request(self, op, req, seed=None, callback=None, suite=SUITE_SHA256):
        """Device queues: builds the ABI item of one request, shaped as for the
        batch helpers (sign_batch ... proof_verify_batch), and queues it on the
        queue of operation op (OP_*) under `suite`; the receiver's output() is
        the signature or proof once replied."""
        if self._processor is not None:
            raise ValueError("enqueue_request needs a device queue")
        if suite not in (SUITE_SHA256, SUITE_SHAKE256) or not 0 <= op < 4:
            raise ValueError("unknown operation or ciphersuite")
        k = _Keep()
        buf = None
        if op == OP_SIGN:
            sk, pk, hdr, msgs = req
            ob, buf = k.out(80)
            items = (SignItem * 1)()
            items[0] = SignItem(k.bytes(sk), k.bytes(pk), k.bytes(hdr), k.slices(msgs), len(msgs), ob)
        elif op == OP_PROOF_GEN:
            items, bufs = _proof_gen_items(k, [req])
            buf = bufs[0]
        else:
            items = _op_items(op, [req], k)
        rec = self.enqueue(serve_queue(op, suite), items[0], seed, callback)
        rec._attach(k, items, buf, op)
        return rec

    def snapshot(self, queue=-1, counts_len=None):
        """The batcher's metrics (BatcherSnapshot, batcher.rs:86-97) of one queue,
        or of all with queue -1; batch_size_counts has counts_len entries
        (default: the largest max_batch_items + 1)."""
        if counts_len is None:
            qs = [queue] if queue >= 0 else range(SERVE_MAX_QUEUES)
            counts_len = max(self.config(q)["max_batch_items"] for q in qs) + 1
        snap = ServeSnapshot()
        counts = (ctypes.c_uint64 * max(1, counts_len))()
        rc = self._lib.cubbs_bbs_gpu_serve_snapshot(self._handle, queue, ctypes.byref(snap), counts,
                                                    ctypes.c_size_t(counts_len))
        if rc:
            raise ValueError(f"serve_snapshot returned {rc}")
        out = {f: getattr(snap, f) for f, _ in ServeSnapshot._fields_}
        out["batch_size_counts"] = list(counts)[:counts_len]
        return out

    def close(self):
        """Serves what is queued, then frees the native queue."""
        if self._handle:
            self._lib.cubbs_bbs_gpu_serve_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


def bench_device_steps(op, reqs, warmup, steps, seeds=None):
    """Replays the device pipeline of one packed batch (inputs resident in HBM).
    Returns (per-step ms list, kernel launches per step, per-item (code, value), stage breakdown)."""
    k = _Keep()
    items = _op_items(op, reqs, k)
    n = len(reqs)
    ms = (ctypes.c_float * steps)()
    launches = ctypes.c_int32(0)
    res = (Result * n)()
    fn = lib().cubbs_bbs_gpu_bench_device_steps_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                   ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    sb = ctypes.create_string_buffer(b"".join(seeds), 32 * n) if seeds is not None else None
    rc = fn(ABI_VERSION, op, ctypes.cast(items, ctypes.c_void_p), n,
            ctypes.cast(sb, ctypes.c_void_p) if sb is not None else None, warmup, steps,
            ctypes.cast(ms, ctypes.c_void_p), ctypes.cast(ctypes.pointer(launches), ctypes.c_void_p),
            ctypes.cast(res, ctypes.c_void_p))
    if rc:
        raise RuntimeError(f"bench_device_steps returned {rc}")
    names = ctypes.create_string_buffer(32 * 16)
    sms = (ctypes.c_float * 16)()
    fs = lib().cubbs_bbs_gpu_bench_stages_v2
    fs.restype = ctypes.c_int32
    fs.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]
    cnt = fs(ctypes.cast(names, ctypes.c_void_p), ctypes.cast(sms, ctypes.c_void_p), 16)
    stages = [(names.raw[32 * j:32 * j + 32].split(b"\0")[0].decode(), sms[j]) for j in range(cnt)]
    return list(ms), launches.value, [(res[i].code, res[i].value) for i in range(n)], stages


def last_transfer_bytes():
    h2d, d2h = ctypes.c_uint64(0), ctypes.c_uint64(0)
    fn = lib().cubbs_bbs_gpu_last_transfer_bytes_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    fn(ctypes.cast(ctypes.pointer(h2d), ctypes.c_void_p), ctypes.cast(ctypes.pointer(d2h), ctypes.c_void_p))
    return h2d.value, d2h.value


def int_peaks():
    """Measured (1e12 IMAD/s, 1e9 Fp products/s) on the current device."""
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    fn = lib().cubbs_bbs_gpu_int_peaks_v2
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    if fn(ctypes.cast(ctypes.pointer(a), ctypes.c_void_p), ctypes.cast(ctypes.pointer(b), ctypes.c_void_p)):
        raise RuntimeError("int_peaks failed")
    return a.value, b.value


PAIRING_PROGRAMS = ["DBL", "ADD", "DBL1", "ADD1", "MUL_F_F_X", "CONJ_F", "INV_U_F", "EASY1_T", "EASY2_T",
                    "COPY_R_T", "COPY_R_A", "COPY_R_X", "CYCLO_R", "MUL_R_R_T", "MUL_R_R_A", "MUL_R_R_X", "S1_A",
                    "S2_A", "S3_A", "S4_X", "S5_R", "MUL_R_R_CA"]


def pairing_probe(wide=False):
    """SM cycles of one run of each pairing program on a lone team (one warp, or
    two with wide=True): {program name: cycles}."""
    buf = (ctypes.c_double * 64)()
    name = "cubbs_bbs_gpu_pairing_probe_wide_for_test_v2" if wide else "cubbs_bbs_gpu_pairing_probe_for_test_v2"
    fn = getattr(lib(), name)
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    n = fn(ctypes.cast(buf, ctypes.c_void_p), 64)
    if n != len(PAIRING_PROGRAMS):
        raise RuntimeError(f"{name} returned {n}")
    return {k: buf[i] for i, k in enumerate(PAIRING_PROGRAMS)}


def prepared_call(op, reqs):
    """Builds the ABI item array once and returns a function that performs one
    synchronous batch call on it (the caller's data stays as built)."""
    k = _Keep()
    items = _op_items(op, reqs, k)
    n = len(reqs)
    res = (Result * n)()
    name = {OP_SIGN: "cubbs_bbs_gpu_sign_batch_v2", OP_VERIFY: "cubbs_bbs_gpu_verify_batch_v2",
            OP_PROOF_GEN: "cubbs_bbs_gpu_proof_gen_batch_v2",
            OP_PROOF_VERIFY: "cubbs_bbs_gpu_proof_verify_batch_v2"}[op]
    fn = getattr(lib(), name)
    ip, rp = ctypes.cast(items, ctypes.c_void_p), ctypes.cast(res, ctypes.c_void_p)
    import numpy as np
    view = np.frombuffer(res, dtype=np.dtype({"names": ["code", "value"], "formats": ["<i4", "u1"],
                                              "offsets": [0, 4], "itemsize": ctypes.sizeof(Result)}))

    def call():
        rc = fn(ABI_VERSION, ip, n, rp)
        if rc:
            raise RuntimeError(f"{name} returned {rc}")
        _ = k  # keep the buffers alive with the closure
        return list(zip(view["code"].tolist(), view["value"].tolist()))
    return call


# ----------------------------------------------------------------------------- bbs-2023 proofValue codec
# Mirrors crates/cubbs-bbs-proofvalue/src/lib.rs (serialize_base / parse_base /
# serialize_derived / parse_derived) over the library's C codec.
PROOFVALUE_ERRORS = {10: "InvalidMultibasePrefix", 11: "InvalidCborPrefix", 12: "InvalidBaseProof",
                     13: "InvalidDerivedProof", 14: "Base64", 15: "Cbor"}


class ProofValueError(ValueError):
    def __init__(self, code):
        super().__init__(PROOFVALUE_ERRORS.get(code, f"code {code}"))
        self.code = code
        self.kind = PROOFVALUE_ERRORS.get(code)


def _pv_text_out(fn, item):
    """Runs a serialize entry point, growing the text buffer once if needed."""
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    need = ctypes.c_size_t(0)
    cap = 4096
    while True:
        buf = ctypes.create_string_buffer(cap)
        rc = fn(ABI_VERSION, ctypes.cast(ctypes.pointer(item), ctypes.c_void_p), ctypes.cast(buf, ctypes.c_void_p),
                cap, ctypes.cast(ctypes.pointer(need), ctypes.c_void_p))
        if rc == ERR_INSUFFICIENT_OUTPUT and need.value > cap:
            cap = need.value
            continue
        if rc:
            raise ProofValueError(rc)
        return buf.raw[:need.value].decode("ascii")


def _parse_u64_like_rust(text):
    body = text[1:] if text.startswith("+") else text
    if not body or not all("0" <= ch <= "9" for ch in body) or int(body) >= 1 << 64:
        raise ProofValueError(13)
    return int(body)


def proofvalue_serialize_base(bbs_signature, bbs_header, public_key, hmac_key, mandatory_pointers):
    """Base proof -> 'u2V0C...' (lib.rs:76-87)."""
    k = _Keep()
    ptrs = [p.encode("utf-8") for p in mandatory_pointers]
    item = ProofValueBase(k.bytes(bbs_signature), k.bytes(bbs_header), k.bytes(public_key), k.bytes(hmac_key),
                          k.slices(ptrs) if ptrs else None, len(ptrs))
    return _pv_text_out(lib().cubbs_bbs_proofvalue_serialize_base_v2, item)


def proofvalue_serialize_derived(bbs_proof, label_map, mandatory_indexes, selective_indexes, presentation_header):
    """Derived proof -> 'u2V0D...' (lib.rs:103-114).  label_map: {'c14n<k>': 'b<v>'};
    keys parsed as the reference does (a later key naming the same number wins)."""
    nums = {}
    for key in sorted(label_map):
        val = label_map[key]
        if not key.startswith("c14n") or not val.startswith("b"):
            raise ProofValueError(13)
        nums[_parse_u64_like_rust(key[4:])] = _parse_u64_like_rust(val[1:])
    k = _Keep()
    keys = sorted(nums)
    U64 = ctypes.c_uint64

    def arr(vals):
        a = (U64 * max(1, len(vals)))(*vals)
        k.refs.append(a)
        return ctypes.cast(a, ctypes.c_void_p)
    item = ProofValueDerived(k.bytes(bbs_proof), arr(keys), arr([nums[x] for x in keys]), len(keys),
                             arr(mandatory_indexes), len(mandatory_indexes), arr(selective_indexes),
                             len(selective_indexes), k.bytes(presentation_header))
    return _pv_text_out(lib().cubbs_bbs_proofvalue_serialize_derived_v2, item)


def _pv_parse(name, text, out):
    raw = text.encode("utf-8") if isinstance(text, str) else text
    cap = 4 * len(raw) + 4096
    arena = ctypes.create_string_buffer(cap)
    used = ctypes.c_size_t(0)
    fn = getattr(lib(), name)
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_void_p]
    rc = fn(ABI_VERSION, raw, len(raw), ctypes.cast(arena, ctypes.c_void_p), cap,
            ctypes.cast(ctypes.pointer(out), ctypes.c_void_p), ctypes.cast(ctypes.pointer(used), ctypes.c_void_p))
    if rc:
        raise ProofValueError(rc)
    return arena


def _slice_bytes(s):
    return ctypes.string_at(s.data, s.len) if s.len else b""


def _u64s(ptr, n):
    return list((ctypes.c_uint64 * n).from_address(ptr)) if n else []


def proofvalue_parse_base(text):
    """'u2V0C...' -> dict of the base proof fields (lib.rs:89-101)."""
    out = ProofValueBase()
    keep = _pv_parse("cubbs_bbs_proofvalue_parse_base_v2", text, out)
    ptrs = (ByteSlice * max(1, out.mandatory_pointer_count)).from_address(out.mandatory_pointers)
    value = {"bbs_signature": _slice_bytes(out.bbs_signature), "bbs_header": _slice_bytes(out.bbs_header),
             "public_key": _slice_bytes(out.public_key), "hmac_key": _slice_bytes(out.hmac_key),
             "mandatory_pointers": [_slice_bytes(ptrs[i]).decode("utf-8")
                                    for i in range(out.mandatory_pointer_count)]}
    del keep
    return value


def proofvalue_parse_derived(text):
    """'u2V0D...' -> dict of the derived proof fields (lib.rs:116-128)."""
    out = ProofValueDerived()
    keep = _pv_parse("cubbs_bbs_proofvalue_parse_derived_v2", text, out)
    keys = _u64s(out.label_keys, out.label_count)
    vals = _u64s(out.label_values, out.label_count)
    value = {"bbs_proof": _slice_bytes(out.bbs_proof),
             "label_map": {"c14n%d" % a: "b%d" % b for a, b in zip(keys, vals)},
             "mandatory_indexes": _u64s(out.mandatory_indexes, out.mandatory_count),
             "selective_indexes": _u64s(out.selective_indexes, out.selective_count),
             "presentation_header": _slice_bytes(out.presentation_header)}
    del keep
    return value


# ----------------------------------------------------------------------------- bbs-2023 input producers
# Mirrors crates/cubbs-vc-di-bbs/src/{hashing,hmac_label,canonical,key,prepared}.rs
# through the library's cubbs_bbs2023_* entry points (host code, plus Sign /
# Verify on the device for the batch issue and verify).  N-Quads are str lines
# ending in "\n" (RDFC output), passed as UTF-8.

BBS2023_ERRORS = {20: "InvalidHmacKeyLength", 21: "InvalidPublicKeyLength", 22: "InvalidMultibasePrefix",
                  23: "InvalidMulticodecHeader", 24: "Base58", 25: "InvalidVerificationMethod"}
BBS2023_HMAC_KEY_LEN = 32


class Bbs2023Error(ValueError):
    def __init__(self, code):
        kind = BBS2023_ERRORS.get(code) or PROOFVALUE_ERRORS.get(code) or f"code {code}"
        super().__init__(kind)
        self.code = code
        self.kind = kind


class LabelEntry(ctypes.Structure):
    _fields_ = [("input", ByteSlice), ("canonical", ByteSlice)]


class Bbs2023IssueItem(ctypes.Structure):
    _fields_ = [("secret_key", ByteSlice), ("public_key", ByteSlice), ("proof_hash", ByteSlice),
                ("mandatory", ctypes.c_void_p), ("mandatory_count", ctypes.c_size_t),
                ("non_mandatory", ctypes.c_void_p), ("non_mandatory_count", ctypes.c_size_t),
                ("hmac_key", ByteSlice), ("mandatory_pointers", ctypes.c_void_p),
                ("mandatory_pointer_count", ctypes.c_size_t), ("proof_value_out", ByteBuffer)]


class Bbs2023VerifyBaseItem(ctypes.Structure):
    _fields_ = [("public_key", ByteSlice), ("proof_hash", ByteSlice), ("mandatory", ctypes.c_void_p),
                ("mandatory_count", ctypes.c_size_t), ("non_mandatory", ctypes.c_void_p),
                ("non_mandatory_count", ctypes.c_size_t), ("proof_value", ByteSlice)]


def _utf8(lines):
    return [s.encode("utf-8") if isinstance(s, str) else bytes(s) for s in lines]


def _labels(k, pairs):
    arr = (LabelEntry * max(1, len(pairs)))()
    for i, (a, b) in enumerate(pairs):
        arr[i] = LabelEntry(k.bytes(a.encode("utf-8")), k.bytes(b.encode("utf-8")))
    k.refs.append(arr)
    return arr


def _b23(name, argtypes):
    fn = getattr(lib(), name)
    fn.restype = ctypes.c_int32
    fn.argtypes = argtypes
    return fn


def bbs2023_hmac_sha256(key, data):
    out = ctypes.create_string_buffer(32)
    P = ctypes.c_void_p
    fn = _b23("cubbs_bbs2023_hmac_sha256_v2", [ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p,
                                               ctypes.c_size_t, P])
    rc = fn(ABI_VERSION, bytes(key), len(key), bytes(data), len(data), ctypes.cast(out, P))
    if rc:
        raise Bbs2023Error(rc)
    return out.raw


def shuffled_bnode_label_map(canonical_id_map, hmac_key):
    """{input label: c14n label} -> {input label: "bN"} (hmac_label.rs:26-50)."""
    k = _Keep()
    pairs = list(canonical_id_map.items())
    arr = _labels(k, pairs)
    idx = (ctypes.c_uint32 * max(1, len(pairs)))()
    P = ctypes.c_void_p
    fn = _b23("cubbs_bbs2023_shuffled_label_map_v2", [ctypes.c_uint32, P, ctypes.c_size_t, ctypes.c_char_p,
                                                      ctypes.c_size_t, P])
    rc = fn(ABI_VERSION, ctypes.cast(arr, P), len(pairs), bytes(hmac_key), len(hmac_key), ctypes.cast(idx, P))
    if rc:
        raise Bbs2023Error(rc)
    return {a: "b%d" % idx[i] for i, (a, _) in enumerate(pairs)}


def canonical_label_map_from_input_map(input_to_canonical, input_to_replacement):
    """{canonical label: replacement} for the inputs both maps hold (canonical.rs:50-62)."""
    return {c: input_to_replacement[i] for i, c in input_to_canonical.items() if i in input_to_replacement}


def relabel_and_sort_canonical_nquads(lines, label_map):
    """Replaces every "_:label" through label_map and sorts the lines bytewise
    (canonical.rs:64-92,130-150)."""
    k = _Keep()
    raw = _utf8(lines)
    sl = k.slices(raw)
    arr = _labels(k, list(label_map.items()))
    out = (ByteSlice * max(1, len(raw)))()
    used = ctypes.c_size_t(0)
    P = ctypes.c_void_p
    fn = _b23("cubbs_bbs2023_relabel_sort_v2", [ctypes.c_uint32, P, ctypes.c_size_t, P, ctypes.c_size_t, P,
                                                ctypes.c_size_t, P, P])
    cap = sum(len(x) for x in raw) * 2 + 64
    while True:
        arena = ctypes.create_string_buffer(cap)
        rc = fn(ABI_VERSION, sl, len(raw), ctypes.cast(arr, P), len(label_map), ctypes.cast(arena, P), cap,
                ctypes.cast(out, P), ctypes.cast(ctypes.pointer(used), P))
        if rc == ERR_INSUFFICIENT_OUTPUT and used.value > cap:
            cap = used.value
            continue
        if rc:
            raise Bbs2023Error(rc)
        return [ctypes.string_at(out[i].data, out[i].len).decode("utf-8", "surrogateescape") if out[i].len else ""
                for i in range(len(raw))]


def bbs2023_header(proof_lines, mandatory):
    """64-byte bbs-2023 header: SHA-256 of the proof lines, then of the mandatory lines (hashing.rs:7-31)."""
    k = _Keep()
    pl, ml = _utf8(proof_lines), _utf8(mandatory)
    out = ctypes.create_string_buffer(64)
    P = ctypes.c_void_p
    fn = _b23("cubbs_bbs2023_header_v2", [ctypes.c_uint32, P, ctypes.c_size_t, P, ctypes.c_size_t, P])
    rc = fn(ABI_VERSION, k.slices(pl), len(pl), k.slices(ml), len(ml), ctypes.cast(out, P))
    if rc:
        raise Bbs2023Error(rc)
    return out.raw


def _key_text(form, pk):
    P = ctypes.c_void_p
    fn = _b23("cubbs_bbs2023_public_key_to_multibase_v2", [ctypes.c_uint32, ctypes.c_int32, ctypes.c_char_p,
                                                           ctypes.c_size_t, P, ctypes.c_size_t, P])
    buf = ctypes.create_string_buffer(512)
    n = ctypes.c_size_t(0)
    rc = fn(ABI_VERSION, form, bytes(pk), len(pk), ctypes.cast(buf, P), 512, ctypes.cast(ctypes.pointer(n), P))
    if rc:
        raise Bbs2023Error(rc)
    return buf.raw[:n.value].decode("ascii")


def _key_parse(form, text):
    P = ctypes.c_void_p
    fn = _b23("cubbs_bbs2023_public_key_from_multibase_v2", [ctypes.c_uint32, ctypes.c_int32, ctypes.c_char_p,
                                                             ctypes.c_size_t, P])
    raw = text.encode("utf-8")
    out = ctypes.create_string_buffer(96)
    rc = fn(ABI_VERSION, form, raw, len(raw), ctypes.cast(out, P))
    if rc:
        raise Bbs2023Error(rc)
    return out.raw


def public_key_to_multibase(pk):
    return _key_text(0, pk)


def did_key_from_public_key(pk):
    return _key_text(1, pk)


def verification_method_from_public_key(pk):
    return _key_text(2, pk)


def public_key_from_multibase(text):
    return _key_parse(0, text)


def public_key_from_did_key(text):
    return _key_parse(1, text)


def public_key_from_verification_method(text):
    return _key_parse(2, text)


def bbs2023_issue_base_proof_batch(items):
    """items: (secret_key, public_key, proof_hash (32 B), mandatory lines, non-mandatory lines,
    hmac_key, mandatory_pointers) -> [(code, proofValue text or None)] (prepared.rs:335-421)."""
    k = _Keep()
    arr = (Bbs2023IssueItem * max(1, len(items)))()
    bufs = []
    for i, (sk, pk, ph, mand, non, hk, ptrs) in enumerate(items):
        m, nm = _utf8(mand), _utf8(non)
        pp = [p.encode("utf-8") for p in ptrs]
        cap = 4 * (80 + 64 + 96 + 32 + sum(len(p) + 9 for p in pp)) // 3 + 64
        ob, buf = k.out(cap)
        bufs.append(buf)
        arr[i] = Bbs2023IssueItem(k.bytes(sk), k.bytes(pk), k.bytes(ph), k.slices(m), len(m), k.slices(nm), len(nm),
                                  k.bytes(hk), k.slices(pp), len(pp), ob)
    res = (Result * max(1, len(items)))()
    P = ctypes.c_void_p
    fn = _b23("cubbs_bbs2023_issue_base_proof_batch_v2", [ctypes.c_uint32, P, ctypes.c_size_t, P])
    rc = fn(ABI_VERSION, ctypes.cast(arr, P), len(items), ctypes.cast(res, P))
    if rc:
        raise RuntimeError(f"issue_base_proof_batch returned {rc}")
    return [(res[i].code, bufs[i].raw[:arr[i].proof_value_out.len].decode("ascii") if res[i].code == 0 else None)
            for i in range(len(items))]


def bbs2023_verify_base_proof_batch(items):
    """items: (public_key, proof_hash, mandatory lines, non-mandatory lines, proofValue text)
    -> [(code, valid)] (prepared.rs:423-513)."""
    k = _Keep()
    arr = (Bbs2023VerifyBaseItem * max(1, len(items)))()
    for i, (pk, ph, mand, non, text) in enumerate(items):
        m, nm = _utf8(mand), _utf8(non)
        arr[i] = Bbs2023VerifyBaseItem(k.bytes(pk), k.bytes(ph), k.slices(m), len(m), k.slices(nm), len(nm),
                                       k.bytes(text.encode("utf-8")))
    res = (Result * max(1, len(items)))()
    P = ctypes.c_void_p
    fn = _b23("cubbs_bbs2023_verify_base_proof_batch_v2", [ctypes.c_uint32, P, ctypes.c_size_t, P])
    rc = fn(ABI_VERSION, ctypes.cast(arr, P), len(items), ctypes.cast(res, P))
    if rc:
        raise RuntimeError(f"verify_base_proof_batch returned {rc}")
    return [(res[i].code, bool(res[i].value)) for i in range(len(items))]
