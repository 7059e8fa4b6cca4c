"""Regenerate tests/golden/cfrg_bls12381_sha256.json and
tests/golden/cfrg_bls12381_shake256.json from the reference tree.

The reference's known-answer data for the BBS hot path lives in
  CFRG-IETF-BBS/fixture_data/bls12-381-sha-256/   (CFRG draft fixtures)
  CFRG-IETF-BBS/fixture_data/bls12-381-shake-256/ (the same for the SHAKE-256 suite)
  native/cuda/tests/sha256_smoke.cpp:25-37          (SHA-256 strings)
  native/cuda/tests/prepare_b_smoke.cpp:58-86       (6-term B-MSM and its expected B)
This script reads those files as data and writes one compact JSON fixture so
that the test suite does not need the reference tree at run time.

Usage: python tests/golden/make_golden.py /path/to/reference
"""
import json
import pathlib
import re
import sys


def fixtures(fx: pathlib.Path) -> dict:
    out = {}
    for name in ["h2s", "MapMessageToScalarAsHash", "generators", "mockedRng", "keypair"]:
        out[name] = json.loads((fx / f"{name}.json").read_text())
    out["signature"] = [json.loads(p.read_text()) for p in sorted((fx / "signature").glob("*.json"))]
    out["proof"] = [json.loads(p.read_text()) for p in sorted((fx / "proof").glob("*.json"))]
    return out


def main(ref_root: str) -> None:
    ref = pathlib.Path(ref_root)
    out = fixtures(ref / "CFRG-IETF-BBS" / "fixture_data" / "bls12-381-sha-256")

    sha_src = (ref / "native" / "cuda" / "tests" / "sha256_smoke.cpp").read_text()
    block = sha_src[sha_src.index("messages = {"):sha_src.index("std::vector<uint8_t> packed")]
    msgs_part, exp_part = block.split("expected = {")
    out["sha256_kat"] = {
        "messages": re.findall(r'"([^"]*)"', msgs_part),
        "digests": re.findall(r'"([0-9a-f]{64})"', exp_part),
    }

    pb_src = (ref / "native" / "cuda" / "tests" / "prepare_b_smoke.cpp").read_text()

    def hexes(after: str, before: str):
        seg = pb_src[pb_src.index(after):pb_src.index(before, pb_src.index(after))]
        return re.findall(r'"([0-9a-f]+)"', seg)

    out["prepare_b_kat"] = {
        "public_key": hexes("public_key = hex_to_bytes(", ";")[0],
        "header": hexes("header = hex_to_bytes(", ";")[0],
        "message_scalars": hexes("scalars = {", "};"),
        "expected_b": hexes("expected_b =", ";")[0],
        "msm_points": hexes("msm_points = {", "};"),
        "msm_scalars": hexes("msm_scalars = {", "};"),
    }
    dst = pathlib.Path(__file__).with_name("cfrg_bls12381_sha256.json")
    dst.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"wrote {dst} ({dst.stat().st_size} bytes)")
    shake = fixtures(ref / "CFRG-IETF-BBS" / "fixture_data" / "bls12-381-shake-256")
    dst = pathlib.Path(__file__).with_name("cfrg_bls12381_shake256.json")
    dst.write_text(json.dumps(shake, indent=1, sort_keys=True) + "\n")
    print(f"wrote {dst} ({dst.stat().st_size} bytes)")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
