"""The drop-in boundary, pinned: this repository's include/cubbs_bbs_gpu_abi.h
has every struct of the reference header with the same size, alignment and
field offsets, the same constants, and every reference prototype with the same
parameter and return types (tests/golden/abi_layout.json, written from the
reference header by tests/golden/make_abi_layout.py).  Also: every symbol the
library exports is declared in the ABI header or the test header.  CPU only."""
import ctypes
import json
import re
import subprocess
import sys

import pytest

from conftest import ROOT, load_package

sys.path.insert(0, str(ROOT / "tests" / "golden"))
import abi_layout  # noqa: E402

GOLDEN = json.loads((ROOT / "tests" / "golden" / "abi_layout.json").read_text())
HEADER = ROOT / "include" / "cubbs_bbs_gpu_abi.h"
TEST_HEADER = ROOT / "include" / "cubbs_bbs_gpu_test.h"


def test_struct_layouts_match_reference():
    structs, _, _ = abi_layout.parse(HEADER.read_text())
    for name, fields in GOLDEN["fields"].items():
        assert name in structs, f"{name} missing"
        assert structs[name] == fields, f"{name}: field order {structs[name]} != {fields}"
    mine = abi_layout.measure(HEADER, {n: GOLDEN["fields"][n] for n in GOLDEN["fields"]})
    assert mine == GOLDEN["structs"]


def test_constants_match_reference():
    _, defines, _ = abi_layout.parse(HEADER.read_text())
    for name, value in GOLDEN["defines"].items():
        assert defines.get(name) == value, name


def test_prototypes_match_reference():
    ok, err = abi_layout.check_prototypes(HEADER, GOLDEN["prototypes"])
    assert ok, err


def test_prototype_check_catches_a_changed_type(tmp_path):
    """The prototype check fails when a parameter type differs (a planted change
    in a copy of the header)."""
    text = HEADER.read_text().replace(
        "int32_t cubbs_bbs_gpu_g1_add_batch_v2(uint32_t abi_version,",
        "int32_t cubbs_bbs_gpu_g1_add_batch_v2(uint64_t abi_version,")
    assert "uint64_t abi_version" in text
    bad = tmp_path / "cubbs_bbs_gpu_abi.h"
    bad.write_text(text)
    ok, _ = abi_layout.check_prototypes(bad, GOLDEN["prototypes"])
    assert not ok


def test_test_header_compiles_as_c_and_cpp(tmp_path):
    src = tmp_path / "t.c"
    src.write_text(f'#include "{TEST_HEADER}"\nint main(void) {{ return 0; }}\n')
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-c", str(src), "-o", str(tmp_path / "t.o")], check=True)
    cpp = tmp_path / "t.cpp"
    cpp.write_text(src.read_text())
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-c", str(cpp), "-o", str(tmp_path / "u.o")], check=True)


def _declared(path):
    return set(re.findall(r"\b(cubbs_bbs\w+)\s*\(", path.read_text()))


def test_every_export_is_declared():
    """Each exported symbol is declared in the ABI header or in the test header
    (test, benchmark and tuning exports), and each declaration is exported."""
    pkg = load_package()
    path = pkg.build()
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln and "cubbs_" in ln}
    declared = _declared(HEADER) | _declared(TEST_HEADER)
    assert exported - declared == set(), sorted(exported - declared)
    assert declared - exported == set(), sorted(declared - exported)
    assert not (_declared(HEADER) & _declared(TEST_HEADER))
