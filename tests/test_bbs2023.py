"""The bbs-2023 input producers of the library (C ABI, host code) against the
reference's own tests (crates/cubbs-vc-di-bbs/src/{hashing,hmac_label,
canonical,key}.rs), its test data (tests/golden/bbs2023.json) and the oracle's
restatement on seeded inputs.  CPU only."""
import hashlib
import json
import random

import pytest

from conftest import ROOT, load_package
from oracle import bbs2023_oracle as O

GOLDEN = json.loads((ROOT / "tests" / "golden" / "bbs2023.json").read_text())


@pytest.fixture(scope="module")
def pkg():
    p = load_package()
    p.build()
    return p


def test_mandatory_hash_concatenates_without_separators(pkg):
    # hashing.rs:36-42
    assert pkg.bbs2023_header([], ["ab", "c"]) == pkg.bbs2023_header([], ["a", "bc"])


def test_header_is_proof_hash_then_mandatory_hash(pkg):
    # hashing.rs:44-50
    h = pkg.bbs2023_header(["p1\n", "p2\n"], ["m\n"])
    assert len(h) == 64
    assert h[:32] == hashlib.sha256(b"p1\np2\n").digest() and h[32:] == hashlib.sha256(b"m\n").digest()
    assert h == O.bbs_header(O.hash_joined_strings(["p1\n", "p2\n"]), O.hash_joined_strings(["m\n"]))


def test_shuffled_map_is_deterministic_and_uses_b_labels(pkg):
    # hmac_label.rs:56-69
    m = {"alice": "c14n0", "bob": "c14n1", "carol": "c14n2"}
    one = pkg.shuffled_bnode_label_map(m, bytes([9] * 32))
    assert one == pkg.shuffled_bnode_label_map(m, bytes([9] * 32))
    assert len(one) == 3 and all(v.startswith("b") for v in one.values())
    assert one == O.shuffled_bnode_label_map(m, bytes([9] * 32))


@pytest.mark.parametrize("seed", range(8))
def test_hmac_and_label_map_match_oracle(pkg, seed):
    rng = random.Random(seed)
    for klen in (0, 1, 32, 64, 65, 200):
        key = bytes(rng.randrange(256) for _ in range(klen))
        data = bytes(rng.randrange(256) for _ in range(rng.randrange(0, 300)))
        assert pkg.bbs2023_hmac_sha256(key, data) == O.hmac_sha256(key, data)
    m = {"e%d" % i: "c14n%d" % i for i in range(rng.randrange(0, 40))}
    key = bytes(rng.randrange(256) for _ in range(32))
    got = pkg.shuffled_bnode_label_map(m, key)
    assert got == O.shuffled_bnode_label_map(m, key)
    assert sorted(got.values(), key=lambda b: int(b[1:])) == ["b%d" % i for i in range(len(m))]


def test_relabels_blank_nodes_and_sorts_lines(pkg):
    # canonical.rs:140-157
    g = GOLDEN["relabel"]
    assert pkg.relabel_and_sort_canonical_nquads(g["lines"], g["label_map"]) == g["expected"]
    assert O.relabel_and_sort_canonical_nquads(g["lines"], g["label_map"]) == g["expected"]


def test_converts_input_label_map_to_canonical_label_map(pkg):
    # canonical.rs:159-177
    g = GOLDEN["label_map_conversion"]
    got = pkg.canonical_label_map_from_input_map(dict(g["input_to_canonical"]), dict(g["input_to_replacement"]))
    assert got == dict(g["expected"])
    assert O.canonical_label_map_from_input_map(dict(g["input_to_canonical"]),
                                                dict(g["input_to_replacement"])) == dict(g["expected"])


@pytest.mark.parametrize("seed", range(6))
def test_relabel_matches_oracle(pkg, seed):
    """Labels up to any Unicode whitespace (tabs, NBSP, U+2003, U+3000 ...), "_:"
    inside literals, labels missing from the map, lines without blank nodes,
    non-ASCII text and sorting by bytes."""
    rng = random.Random(seed)
    ws = [" ", "\t", " ", " ", "　", "\u0085", "\x0b"]
    labels = ["c14n%d" % i for i in range(12)] + ["x", "ünï", "a_:b"]
    lines = []
    for _ in range(rng.randrange(1, 30)):
        parts = []
        for _ in range(rng.randrange(1, 5)):
            kind = rng.randrange(4)
            if kind == 0:
                parts.append("_:" + rng.choice(labels))
            elif kind == 1:
                parts.append("<urn:%s>" % rng.choice(["p", "é", "q_:r"]))
            elif kind == 2:
                parts.append('"lit _:%s"' % rng.choice(labels))
            else:
                parts.append("_:")
        lines.append(rng.choice(ws).join(parts) + " .\n")
    m = {lab: "b%d" % rng.randrange(100) for lab in labels if rng.random() < 0.7}
    assert pkg.relabel_and_sort_canonical_nquads(lines, m) == O.relabel_and_sort_canonical_nquads(lines, m)


def test_digital_bazaar_multikey_vector(pkg):
    # key.rs:105-111
    mk = GOLDEN["multikey_vector"]
    pk = pkg.public_key_from_multibase(mk)
    assert len(pk) == 96 and pkg.public_key_to_multibase(pk) == mk
    assert pk == O.public_key_from_multibase(mk)
    did = pkg.did_key_from_public_key(pk)
    vm = pkg.verification_method_from_public_key(pk)
    assert did == "did:key:" + mk and vm == did + "#" + mk
    assert pkg.public_key_from_did_key(did) == pk
    assert pkg.public_key_from_verification_method(vm) == pk
    assert pkg.public_key_from_verification_method(did) == pk


@pytest.mark.parametrize("seed", range(6))
def test_multikey_round_trips_match_oracle(pkg, seed):
    rng = random.Random(seed)
    pk = bytes(rng.randrange(256) for _ in range(96))
    if seed == 0:
        pk = bytes(96)  # leading zero bytes after the multicodec header
    mk = pkg.public_key_to_multibase(pk)
    assert mk == O.public_key_to_multibase(pk)
    assert pkg.public_key_from_multibase(mk) == pk


def _kind(fn, *a):
    with pytest.raises(ValueError) as e:
        fn(*a)
    return e.value.kind


def test_key_errors(pkg):
    mk = GOLDEN["multikey_vector"]
    assert _kind(pkg.public_key_to_multibase, bytes(95)) == "InvalidPublicKeyLength"
    assert _kind(pkg.public_key_from_multibase, mk[1:]) == "InvalidMultibasePrefix"
    assert _kind(pkg.public_key_from_multibase, "z0OIl") == "Base58"
    assert _kind(pkg.public_key_from_multibase, "z" + O.b58encode(bytes([0xEB, 0x02]) + bytes(96))) == \
        "InvalidMulticodecHeader"
    assert _kind(pkg.public_key_from_multibase, "z" + O.b58encode(bytes([0xEB]))) == "InvalidMulticodecHeader"
    assert _kind(pkg.public_key_from_multibase, "z" + O.b58encode(bytes([0xEB, 0x01]) + bytes(95))) == \
        "InvalidPublicKeyLength"
    assert _kind(pkg.public_key_from_did_key, mk) == "InvalidVerificationMethod"
    assert _kind(pkg.public_key_from_verification_method, "did:web:x") == "InvalidVerificationMethod"
    for bad, kind in ((mk[1:], "InvalidMultibasePrefix"), ("z0OIl", "Base58")):
        with pytest.raises(O.KeyError_) as e:
            O.public_key_from_multibase(bad)
        assert e.value.kind == kind
