"""Deterministic synthetic inputs for parity tests (seeded SHA-256 counter DRBG)."""
import hashlib

R_MOD = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def drbg(seed: bytes, label: bytes, i: int, n: int) -> bytes:
    out = b""
    ctr = 0
    while len(out) < n:
        out += hashlib.sha256(seed + label + i.to_bytes(8, "big") + ctr.to_bytes(4, "big")).digest()
        ctr += 1
    return out[:n]


def scalar(seed: bytes, label: bytes, i: int) -> bytes:
    """Uniform Fr scalar (48 DRBG bytes reduced mod r), 32-byte big-endian."""
    v = int.from_bytes(drbg(seed, label, i, 48), "big") % R_MOD
    return v.to_bytes(32, "big")


def keypair(oracle, seed: bytes, i: int = 0):
    sk = oracle.keygen(drbg(seed, b"key", i, 32))
    return sk, oracle.sk_to_pk(sk)


def messages(seed: bytes, tag: int, L: int, size: int):
    return [drbg(seed, b"msg%d" % tag, j, size) for j in range(L)]


def disclosed_subset(seed: bytes, tag: int, L: int, R: int):
    order = sorted(range(L), key=lambda j: drbg(seed, b"disc%d" % tag, j, 8))
    return sorted(order[:R])
