"""Regenerate tests/golden/bbs2023.json from the reference tree.

The reference's own test data for the bbs-2023 input producers:
  crates/cubbs-vc-di-bbs/src/key.rs       (a Digital Bazaar BBS Multikey vector)
  crates/cubbs-vc-di-bbs/src/canonical.rs (relabel-and-sort lines, label maps
                                            and the expected output)
This script reads those files as text and writes them as one JSON fixture, so
that the test suite does not need the reference tree at run time.

Usage: python tests/golden/make_bbs2023_golden.py /path/to/reference
"""
import json
import pathlib
import re
import sys


def rust_strings(block: str):
    """The "..." string literals of a Rust block, with \\n and \\" unescaped."""
    return [s.encode().decode("unicode_escape") for s in re.findall(r'"((?:[^"\\]|\\.)*)"', block)]


def main(ref_root: str) -> None:
    src = pathlib.Path(ref_root) / "crates" / "cubbs-vc-di-bbs" / "src"
    key = (src / "key.rs").read_text()
    fn = key[key.index("fn parses_digital_bazaar_bbs_multikey_vector"):]
    multikey = re.search(r'let multibase = "(z[1-9A-HJ-NP-Za-km-z]+)"', fn).group(1)

    canon = (src / "canonical.rs").read_text()
    t = canon[canon.index("fn relabels_blank_nodes_and_sorts_lines"):]
    t = t[:t.index("#[test]")] if "#[test]" in t else t
    lines_block = t[t.index("let lines = vec!["):t.index("];")]
    map_block = t[t.index("let label_map = BTreeMap::from(["):t.index("]);")]
    expect_block = t[t.index("vec![", t.index("assert_eq!(")):]
    expect_block = expect_block[:expect_block.index("]")]
    m = rust_strings(map_block)

    c = canon[canon.index("fn converts_input_label_map_to_canonical_label_map"):]
    blocks = re.findall(r"BTreeMap::from\(\[(.*?)\]\)", c, re.S)
    to_pairs = lambda b: [list(p) for p in re.findall(r'\("([^"]*)"\.to_owned\(\),\s*"([^"]*)"\.to_owned\(\)\)', b)]

    out = {
        "multikey_vector": multikey,
        "relabel": {"lines": rust_strings(lines_block), "label_map": dict(zip(m[0::2], m[1::2])),
                    "expected": rust_strings(expect_block)},
        "label_map_conversion": {"input_to_canonical": to_pairs(blocks[0]),
                                 "input_to_replacement": to_pairs(blocks[1]), "expected": to_pairs(blocks[2])},
    }
    dst = pathlib.Path(__file__).resolve().parent / "bbs2023.json"
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
