"""Writes bbs_dst.cuh: the domain-separation strings and P1 of the two BBS
ciphersuites (crates/cubbs-bbs-protocol/src/bbsplus/ciphersuites.rs:21-79) as
constant-memory byte arrays, and Suite<S> accessors over them.

    python gen_bbs_dst.py
"""
import pathlib

SUITES = {
    0: ("BBS_BLS12381G1_XMD:SHA-256_SSWU_RO_H2G_HM2S_",
        "a8ce256102840821a3e94ea9025e4662b205762f9776b3a766c872b948f1fd225e7c59698588e70d11406d161b4e28c9"),
    1: ("BBS_BLS12381G1_XOF:SHAKE-256_SSWU_RO_H2G_HM2S_",
        "8929dfbc7e6642c4ed9cba0856e493f8b9d7d5fcb0c31ef8fdcd34d50648a56c795e106e9eada6e0bda386b414150755"),
}
SUFFIX = {  # name -> (suffix appended to API_ID; None: API_ID itself)
    "API_ID": None,
    "DST_H2S": "H2S_",
    "DST_MAP": "MAP_MSG_TO_SCALAR_AS_HASH_",
    "DST_MOCK": "MOCK_RANDOM_SCALARS_DST_",
    "DST_GEN_SEED": "SIG_GENERATOR_SEED_",
    "DST_GEN": "SIG_GENERATOR_DST_",
    "GEN_SEED": "MESSAGE_GENERATOR_SEED",
}


def arr(name, data):
    body = ", ".join(f"0x{b:02x}" for b in data)
    return [f"#define {name}_LEN {len(data)}",
            f"__device__ __constant__ static const uint8_t {name}[{len(data)}] = {{{body}}};"]


def main():
    lines = ["// GENERATED by gen_bbs_dst.py -- do not edit by hand.",
             "// Domain-separation strings and P1 of the BBS ciphersuites",
             "// (crates/cubbs-bbs-protocol/src/bbsplus/ciphersuites.rs:21-79) in constant memory:",
             "// suite 0 BBS_BLS12381G1_XMD:SHA-256_SSWU_RO_ (names without a suffix),",
             "// suite 1 BBS_BLS12381G1_XOF:SHAKE-256_SSWU_RO_ (names ending in _XOF).",
             "#pragma once",
             "#include <stdint.h>",
             ""]
    for suite, (api, p1) in SUITES.items():
        tag = "" if suite == 0 else "_XOF"
        for name, suf in SUFFIX.items():
            s = api if suf is None else api + suf
            lines += arr(name + tag, s.encode())
        lines += arr("P1_COMPRESSED" + tag, bytes.fromhex(p1))
        lines.append("")
    lines += ["// Suite<S>: the strings of suite S (used by the templated hash kernels).",
              "template <int S> struct SuiteDst;"]
    for suite in SUITES:
        tag = "" if suite == 0 else "_XOF"
        lines.append(f"template <> struct SuiteDst<{suite}> {{")
        for name in list(SUFFIX) + ["P1_COMPRESSED"]:
            lname = name.lower()
            lines.append(f"  static __device__ __forceinline__ const uint8_t *{lname}() {{ return {name}{tag}; }}")
            lines.append(f"  static constexpr uint32_t {lname}_len = {name}{tag}_LEN;")
        lines.append("};")
    lines.append("")
    out = pathlib.Path(__file__).with_name("bbs_dst.cuh")
    out.write_text("\n".join(lines))
    print("wrote", out)


if __name__ == "__main__":
    main()
