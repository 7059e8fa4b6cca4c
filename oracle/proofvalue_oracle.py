"""CPU oracle of the W3C bbs-2023 proofValue codec (TEST INFRASTRUCTURE ONLY:
imported by tests/ as the checker, never by the product).

Restates crates/cubbs-bbs-proofvalue/src/lib.rs:1-220 and the encoding of
its third-party serializer (serde_cbor 0.11: a tuple struct is a definite
CBOR array, Vec<u8> under serde_bytes a byte string, String a text string,
BTreeMap<u64, u64> a definite map in ascending key order, every length and
integer in its shortest form) with the multibase base64url-no-pad wrapper
(base64 0.22 URL_SAFE_NO_PAD: no padding accepted, zero trailing bits).
Written from those rules with Python's standard library only.

Parity: the reference's own tests pin only the prefixes 'u2V0C' / 'u2V0D'
and round trips (lib.rs:208-218); no golden proofValue string exists in the
reference tree, so byte-level parity of the encoding rests on this
restatement of the published CBOR rules (parity unpinned beyond that).
"""
import base64

PREFIX_BASE = bytes([0xD9, 0x5D, 0x02])
PREFIX_DERIVED = bytes([0xD9, 0x5D, 0x03])


class ProofValueError(ValueError):
    """kind: multibase_prefix, cbor_prefix, invalid_base, invalid_derived, base64, cbor."""

    def __init__(self, kind):
        super().__init__(kind)
        self.kind = kind


def _head(major, v):
    if v < 24:
        return bytes([major << 5 | v])
    for ai, n in ((24, 1), (25, 2), (26, 4), (27, 8)):
        if v < 1 << (8 * n):
            return bytes([major << 5 | ai]) + v.to_bytes(n, "big")
    raise ValueError("integer too large")


def _bstr(b):
    return _head(2, len(b)) + bytes(b)


def _tstr(s):
    raw = s.encode("utf-8")
    return _head(3, len(raw)) + raw


def _uint(v):
    return _head(0, v)


def _wrap(prefix, payload):
    return "u" + base64.urlsafe_b64encode(prefix + payload).decode().rstrip("=")


def parse_rust_u64(text):
    """Rust's u64::from_str: an optional '+', then one or more ASCII digits, below 2^64."""
    body = text[1:] if text.startswith("+") else text
    if not body or not all("0" <= ch <= "9" for ch in body):
        raise ProofValueError("invalid_derived")
    v = int(body)
    if v >= 1 << 64:
        raise ProofValueError("invalid_derived")
    return v


def compress_label_map(label_map):
    """{'c14n<k>': 'b<v>'} -> {k: v} (lib.rs:177-199): keys in the string map's
    order, a later key with the same number replacing an earlier one."""
    out = {}
    for k in sorted(label_map):
        v = label_map[k]
        if not k.startswith("c14n") or not v.startswith("b"):
            raise ProofValueError("invalid_derived")
        out[parse_rust_u64(k[4:])] = parse_rust_u64(v[1:])
    return out


def serialize_base(sig, header, pk, hmac_key, pointers):
    if len(sig) != 80 or len(header) != 64 or len(pk) != 96 or len(hmac_key) != 32:
        raise ProofValueError("invalid_base")
    payload = _head(4, 5) + _bstr(sig) + _bstr(header) + _bstr(pk) + _bstr(hmac_key)
    payload += _head(4, len(pointers)) + b"".join(_tstr(p) for p in pointers)
    return _wrap(PREFIX_BASE, payload)


def serialize_derived(proof, label_map, mandatory, selective, ph):
    """label_map in the numeric form {k: v}."""
    if not proof:
        raise ProofValueError("invalid_derived")
    payload = _head(4, 5) + _bstr(proof) + _head(5, len(label_map))
    payload += b"".join(_uint(k) + _uint(label_map[k]) for k in sorted(label_map))
    payload += _head(4, len(mandatory)) + b"".join(_uint(x) for x in mandatory)
    payload += _head(4, len(selective)) + b"".join(_uint(x) for x in selective)
    payload += _bstr(ph)
    return _wrap(PREFIX_DERIVED, payload)


class _Reader:
    def __init__(self, b):
        self.b, self.at = b, 0

    def head(self):
        if self.at >= len(self.b):
            raise ProofValueError("cbor")
        first = self.b[self.at]
        self.at += 1
        major, ai = first >> 5, first & 31
        if ai < 24:
            return major, ai
        n = {24: 1, 25: 2, 26: 4, 27: 8}.get(ai)
        if n is None or self.at + n > len(self.b):
            raise ProofValueError("cbor")
        v = int.from_bytes(self.b[self.at:self.at + n], "big")
        self.at += n
        return major, v

    def expect(self, major):
        m, v = self.head()
        if m != major:
            raise ProofValueError("cbor")
        return v

    def string(self, major):
        n = self.expect(major)
        if n > len(self.b) - self.at:
            raise ProofValueError("cbor")
        out = self.b[self.at:self.at + n]
        self.at += n
        return out


def _unwrap(text, prefix):
    if not text.startswith("u"):
        raise ProofValueError("multibase_prefix")
    body = text[1:]
    alphabet = set("ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789-_")
    if len(body) % 4 == 1 or any(ch not in alphabet for ch in body):
        raise ProofValueError("base64")
    raw = base64.urlsafe_b64decode(body + "=" * (-len(body) % 4))
    if base64.urlsafe_b64encode(raw).decode().rstrip("=") != body:  # nonzero trailing bits
        raise ProofValueError("base64")
    if raw[:3] != prefix:
        raise ProofValueError("cbor_prefix")
    return raw[3:]


def parse_base(text):
    r = _Reader(_unwrap(text, PREFIX_BASE))
    if r.expect(4) != 5:
        raise ProofValueError("cbor")
    sig, hdr, pk, hk = (r.string(2) for _ in range(4))
    ptrs = []
    for _ in range(r.expect(4)):
        try:
            ptrs.append(r.string(3).decode("utf-8"))
        except UnicodeDecodeError:
            raise ProofValueError("cbor")
    if r.at != len(r.b):
        raise ProofValueError("cbor")
    if len(sig) != 80 or len(hdr) != 64 or len(pk) != 96 or len(hk) != 32:
        raise ProofValueError("invalid_base")
    return sig, hdr, pk, hk, ptrs


def parse_derived(text):
    r = _Reader(_unwrap(text, PREFIX_DERIVED))
    if r.expect(4) != 5:
        raise ProofValueError("cbor")
    proof = r.string(2)
    labels = {}
    for _ in range(r.expect(5)):
        k = r.expect(0)
        labels[k] = r.expect(0)
    mand = [r.expect(0) for _ in range(r.expect(4))]
    sel = [r.expect(0) for _ in range(r.expect(4))]
    ph = r.string(2)
    if r.at != len(r.b):
        raise ProofValueError("cbor")
    if not proof:
        raise ProofValueError("invalid_derived")
    return proof, labels, mand, sel, ph
