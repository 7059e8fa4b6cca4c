"""CPU oracle of the W3C bbs-2023 input producers (TEST INFRASTRUCTURE ONLY:
imported by tests/ as the checker, never by the product).

Restates, with Python's standard library (hashlib, hmac, base64) and a base58
restatement of its own:
  crates/cubbs-vc-di-bbs/src/hashing.rs:7-31     hash_joined_strings, bbs_header
  crates/cubbs-vc-di-bbs/src/hmac_label.rs:11-50 hmac_sha256, shuffled_bnode_label_map
  crates/cubbs-vc-di-bbs/src/canonical.rs:50-150 label map conversion, relabel and sort
  crates/cubbs-vc-di-bbs/src/key.rs:25-80        Multikey / did:key forms of a G2 public key
  crates/cubbs-vc-di-bbs/src/prepared.rs:335-513 the header and message lowering of issue
                                                  and base verification
The base58btc codec follows the bs58 crate's Bitcoin alphabet.

Pinned by the reference's own test data (tests/golden/bbs2023.json: a Digital
Bazaar Multikey vector, the relabel-and-sort case, the label map conversion);
the hash and HMAC steps rest on Python's hashlib and hmac.
"""
import base64
import hashlib
import hmac

B58 = "123456789ABCDEFGHJKLMNPQRSTUVWXYZabcdefghijkmnopqrstuvwxyz"
MULTICODEC_G2 = bytes([0xEB, 0x01])

# Rust's char::is_whitespace: the Unicode White_Space property
RUST_WHITESPACE = {0x09, 0x0A, 0x0B, 0x0C, 0x0D, 0x20, 0x85, 0xA0, 0x1680, 0x2028, 0x2029, 0x202F, 0x205F,
                   0x3000} | set(range(0x2000, 0x200B))


class KeyError_(ValueError):
    def __init__(self, kind):
        super().__init__(kind)
        self.kind = kind


def hash_joined_strings(lines):
    return hashlib.sha256("".join(lines).encode("utf-8")).digest()


def bbs_header(proof_hash, mandatory_hash):
    return bytes(proof_hash) + bytes(mandatory_hash)


def hmac_sha256(key, data):
    return hmac.new(bytes(key), bytes(data), hashlib.sha256).digest()


def shuffled_bnode_label_map(canonical_id_map, key):
    ids = {inp: "u" + base64.urlsafe_b64encode(hmac_sha256(key, c.encode())).decode().rstrip("=")
           for inp, c in canonical_id_map.items()}
    ranked = sorted(ids.values())
    return {inp: "b%d" % ranked.index(h) for inp, h in ids.items()}


def canonical_label_map_from_input_map(input_to_canonical, input_to_replacement):
    return {c: input_to_replacement[i] for i, c in input_to_canonical.items() if i in input_to_replacement}


def _relabel_line(line, label_map):
    out, rest = [], line
    while True:
        pos = rest.find("_:")
        if pos < 0:
            break
        out.append(rest[:pos + 2])
        end = pos + 2
        while end < len(rest) and ord(rest[end]) not in RUST_WHITESPACE:
            end += 1
        label = rest[pos + 2:end]
        out.append(label_map.get(label, label))
        rest = rest[end:]
    out.append(rest)
    return "".join(out)


def relabel_and_sort_canonical_nquads(lines, label_map):
    return sorted((_relabel_line(x, label_map) for x in lines), key=lambda s: s.encode("utf-8"))


def b58encode(data):
    n = int.from_bytes(data, "big")
    out = ""
    while n:
        n, r = divmod(n, 58)
        out = B58[r] + out
    zeros = len(data) - len(data.lstrip(b"\0"))
    return "1" * zeros + out


def b58decode(text):
    n = 0
    for ch in text:
        if ch not in B58:
            raise KeyError_("Base58")
        n = n * 58 + B58.index(ch)
    ones = len(text) - len(text.lstrip("1"))
    body = n.to_bytes((n.bit_length() + 7) // 8, "big") if n else b""
    return b"\0" * ones + body


def public_key_to_multibase(pk):
    if len(pk) != 96:
        raise KeyError_("InvalidPublicKeyLength")
    return "z" + b58encode(MULTICODEC_G2 + bytes(pk))


def public_key_from_multibase(text):
    if not text.startswith("z"):
        raise KeyError_("InvalidMultibasePrefix")
    raw = b58decode(text[1:])
    if not raw.startswith(MULTICODEC_G2):
        raise KeyError_("InvalidMulticodecHeader")
    if len(raw) - 2 != 96:
        raise KeyError_("InvalidPublicKeyLength")
    return raw[2:]


def did_key_from_public_key(pk):
    return "did:key:" + public_key_to_multibase(pk)


def verification_method_from_public_key(pk):
    mb = public_key_to_multibase(pk)
    return "did:key:%s#%s" % (mb, mb)


def public_key_from_did_key(text):
    if not text.startswith("did:key:"):
        raise KeyError_("InvalidVerificationMethod")
    return public_key_from_multibase(text[len("did:key:"):])


def public_key_from_verification_method(text):
    if "#" in text:
        return public_key_from_multibase(text.split("#", 1)[1])
    return public_key_from_did_key(text)


def issue_lowering(proof_hash, mandatory, non_mandatory):
    """(header, messages) of IssueBaseProofRequest (prepared.rs:335-345)."""
    return bbs_header(proof_hash, hash_joined_strings(mandatory)), [s.encode("utf-8") for s in non_mandatory]
