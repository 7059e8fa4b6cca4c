"""The bbs-2023 proofValue codec of the library (C ABI, host code) against the
reference crate's own tests (crates/cubbs-bbs-proofvalue/src/lib.rs:208-218:
round trips and the 'u2V0C' / 'u2V0D' prefixes) and against the oracle's
restatement of the CBOR and base64url rules, byte for byte; malformed inputs
give the reference's error kinds.  CPU only."""
import base64
import random

import pytest

from conftest import load_package
from oracle import proofvalue_oracle as O



@pytest.fixture(scope="module")
def pv():
    pkg = load_package()
    pkg.build()
    pkg.lib()
    return pkg


def rand_bytes(rng, n):
    return bytes(rng.randrange(256) for _ in range(n))


def test_reference_base_round_trip(pv):
    text = pv.proofvalue_serialize_base(b"\x01" * 80, b"\x02" * 64, b"\x03" * 96, b"\x04" * 32, ["/issuer"])
    assert text.startswith("u2V0C")
    assert pv.proofvalue_parse_base(text) == {"bbs_signature": b"\x01" * 80, "bbs_header": b"\x02" * 64,
                                              "public_key": b"\x03" * 96, "hmac_key": b"\x04" * 32,
                                              "mandatory_pointers": ["/issuer"]}


def test_reference_derived_round_trip(pv):
    value = {"bbs_proof": b"\x01" * 272, "label_map": {"c14n0": "b2", "c14n1": "b0"},
             "mandatory_indexes": [0, 1, 4], "selective_indexes": [2, 3], "presentation_header": b"ph"}
    text = pv.proofvalue_serialize_derived(value["bbs_proof"], value["label_map"], value["mandatory_indexes"],
                                           value["selective_indexes"], value["presentation_header"])
    assert text.startswith("u2V0D")
    assert pv.proofvalue_parse_derived(text) == value


@pytest.mark.parametrize("seed", range(12))
def test_random_values_match_oracle(pv, seed):
    rng = random.Random(seed)
    sig, hdr, pk, hk = (rand_bytes(rng, n) for n in (80, 64, 96, 32))
    ptrs = ["/" + "".join(rng.choice("abcé/xyz0") for _ in range(rng.randrange(0, 30))) for _ in range(rng.randrange(0, 40))]
    text = pv.proofvalue_serialize_base(sig, hdr, pk, hk, ptrs)
    assert text == O.serialize_base(sig, hdr, pk, hk, ptrs)
    assert O.parse_base(text) == (sig, hdr, pk, hk, ptrs)
    assert pv.proofvalue_parse_base(text)["mandatory_pointers"] == ptrs
    proof = rand_bytes(rng, rng.choice((272, 304, 1872, 20000)))
    widths = (0, 23, 24, 255, 256, 65535, 65536, 2**32 - 1, 2**32, 2**64 - 1)
    labels = {rng.choice(widths) if k < 3 else rng.randrange(10**6): rng.randrange(2**40) for k in range(rng.randrange(0, 60))}
    mand = [rng.choice(widths) for _ in range(rng.randrange(0, 50))]
    sel = sorted(rng.sample(range(10**5), rng.randrange(0, 50)))
    ph = rand_bytes(rng, rng.choice((0, 1, 23, 24, 64, 300)))
    lm = {"c14n%d" % k: "b%d" % v for k, v in labels.items()}
    text = pv.proofvalue_serialize_derived(proof, lm, mand, sel, ph)
    assert text == O.serialize_derived(proof, O.compress_label_map(lm), mand, sel, ph)
    assert pv.proofvalue_parse_derived(text) == {"bbs_proof": proof, "label_map": lm, "mandatory_indexes": mand,
                                                  "selective_indexes": sel, "presentation_header": ph}


def _wrap(prefix, payload):
    return "u" + base64.urlsafe_b64encode(prefix + payload).decode().rstrip("=")


def test_decoding_accepts_wider_integers_and_repeated_keys(pv):
    """Lengths and integers in wider forms than needed decode (the reference's
    decoder takes any width); a repeated map key keeps its last value."""
    body = bytes([0x85, 0x59, 0x00, 0x03]) + b"abc" + bytes([0xA2, 0x01, 0x02, 0x01, 0x1A, 0, 0, 0, 9])
    body += bytes([0x82, 0x18, 0x05, 0x1B] + [0] * 7 + [7]) + bytes([0x80, 0x40])
    text = _wrap(O.PREFIX_DERIVED, body)
    want = {"bbs_proof": b"abc", "label_map": {"c14n1": "b9"}, "mandatory_indexes": [5, 7],
            "selective_indexes": [], "presentation_header": b""}
    assert pv.proofvalue_parse_derived(text) == want
    proof, labels, mand, sel, ph = O.parse_derived(text)
    assert (proof, labels, mand, sel, ph) == (b"abc", {1: 9}, [5, 7], [], b"")


def _kind(fn, *args):
    with pytest.raises(Exception) as e:
        fn(*args)
    return e.value.kind


@pytest.mark.parametrize("case,kind", [
    ("x2V0C", "InvalidMultibasePrefix"),
    ("", "InvalidMultibasePrefix"),
    ("u2V0D" + "A" * 8, "InvalidCborPrefix"),
    ("u", "InvalidCborPrefix"),
    ("u2V0C=", "Base64"),
    ("u2V0C+AAA", "Base64"),
    ("u2V0CA", "Base64"),
    ("u2V0CAB", "Base64"),
])
def test_malformed_text(pv, case, kind):
    assert _kind(pv.proofvalue_parse_base, case) == kind
    oracle_kind = {"InvalidMultibasePrefix": "multibase_prefix", "InvalidCborPrefix": "cbor_prefix",
                   "Base64": "base64"}[kind]
    assert _kind(O.parse_base, case) == oracle_kind


def test_malformed_payloads(pv):
    good = O.serialize_base(b"\x01" * 80, b"\x02" * 64, b"\x03" * 96, b"\x04" * 32, ["/a"])
    raw = base64.urlsafe_b64decode(good[1:] + "=" * (-len(good[1:]) % 4))
    payload = raw[3:]
    cases = {
        "trailing": _wrap(O.PREFIX_BASE, payload + b"\x00"),
        "truncated": _wrap(O.PREFIX_BASE, payload[:-1]),
        "four fields": _wrap(O.PREFIX_BASE, bytes([0x84]) + payload[1:payload.index(bytes([0x81]), 200)]),
        "indefinite": _wrap(O.PREFIX_BASE, bytes([0x9F]) + payload[1:] + bytes([0xFF])),
        "bad utf-8": _wrap(O.PREFIX_BASE, payload[:-2] + bytes([0x61, 0xFF])),
    }
    for name, text in cases.items():
        assert _kind(pv.proofvalue_parse_base, text) == "Cbor", name
        assert _kind(O.parse_base, text) == "cbor", name
    bad_len = _wrap(O.PREFIX_BASE, bytes([0x85, 0x41, 0x00]) + payload[1 + 2 + 80:])
    assert _kind(pv.proofvalue_parse_base, bad_len) == "InvalidBaseProof"
    assert _kind(O.parse_base, bad_len) == "invalid_base"
    empty = _wrap(O.PREFIX_DERIVED, bytes([0x85, 0x40, 0xA0, 0x80, 0x80, 0x40]))
    assert _kind(pv.proofvalue_parse_derived, empty) == "InvalidDerivedProof"
    assert _kind(O.parse_derived, empty) == "invalid_derived"


def test_serialize_rejects_what_the_reference_rejects(pv):
    assert _kind(pv.proofvalue_serialize_base, b"\x01" * 79, b"\x02" * 64, b"\x03" * 96, b"\x04" * 32,
                 []) == "InvalidBaseProof"
    assert _kind(pv.proofvalue_serialize_derived, b"", {}, [], [], b"") == "InvalidDerivedProof"
    for bad in ({"c14x0": "b1"}, {"c14n": "b1"}, {"c14n1": "1"}, {"c14n-1": "b1"}, {"c14n1": "b%d" % 2**64}):
        assert _kind(pv.proofvalue_serialize_derived, b"p", bad, [], [], b"") == "InvalidDerivedProof", bad
    # Rust's u64 parse takes a leading '+' and leading zeros; two keys naming one
    # number keep the later one in the string map's (byte) order: '+' < '0'
    text = pv.proofvalue_serialize_derived(b"p", {"c14n+3": "b007", "c14n03": "b5"}, [], [], b"")
    assert pv.proofvalue_parse_derived(text)["label_map"] == {"c14n3": "b5"}
    assert O.compress_label_map({"c14n+3": "b007", "c14n03": "b5"}) == {3: 5}
    text = pv.proofvalue_serialize_derived(b"p", {"c14n+3": "b007"}, [], [], b"")
    assert pv.proofvalue_parse_derived(text)["label_map"] == {"c14n3": "b7"}
