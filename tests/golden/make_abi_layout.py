"""Writes tests/golden/abi_layout.json from the reference's C ABI header
(native/cuda/include/cubbs_bbs_gpu_abi.h): struct sizes, alignments and field
offsets measured with gcc, the #define constants and the function prototypes.
Run in the container that holds the reference checkout:

    python tests/golden/make_abi_layout.py /root/reference
"""
import json
import pathlib
import sys

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import abi_layout  # noqa: E402


def main(ref_root: str) -> None:
    header = pathlib.Path(ref_root) / "native" / "cuda" / "include" / "cubbs_bbs_gpu_abi.h"
    structs, defines, protos = abi_layout.parse(header.read_text())
    layout = abi_layout.measure(header, structs)
    ok, err = abi_layout.check_prototypes(header, protos)
    assert ok, err
    out = {"source": "native/cuda/include/cubbs_bbs_gpu_abi.h", "structs": layout, "fields": structs,
           "defines": defines, "prototypes": protos}
    (HERE / "abi_layout.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"{len(layout)} structs, {len(defines)} constants, {len(protos)} prototypes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
