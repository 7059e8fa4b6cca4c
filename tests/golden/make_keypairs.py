"""Generate tests/golden/keypairs256.json: 256 BBS keypairs for the serving
benchmark (256 device-resident public keys).  KeyGen over 32-byte key material
SHA-256("cubbs-serving-keys" || I2OSP(i, 8)) with the oracle's KeyGen/SkToPk,
which the CFRG keypair fixture pins.  Run from the repository root:
    python tests/golden/make_keypairs.py
"""
import hashlib
import json
import pathlib
import sys

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def main() -> None:
    from oracle import oracle_ctypes as O
    O.lib()
    keys = []
    for i in range(256):
        ikm = hashlib.sha256(b"cubbs-serving-keys" + i.to_bytes(8, "big")).digest()
        sk = O.keygen(ikm)
        keys.append({"sk": sk.hex(), "pk": O.sk_to_pk(sk).hex()})
    dst = pathlib.Path(__file__).with_name("keypairs256.json")
    dst.write_text(json.dumps(keys, indent=0) + "\n")
    print(f"wrote {dst} ({dst.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
