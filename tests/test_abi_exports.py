"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
entry point include/cubbs_bbs_gpu_abi.h declares (CPU only: no compute calls)."""
import ctypes
import re

from conftest import ROOT, load_package


def declared_symbols():
    text = (ROOT / "include" / "cubbs_bbs_gpu_abi.h").read_text()
    return sorted(set(re.findall(r"\b(cubbs_bbs\w+)\s*\(", text)))


def test_header_declares_reference_symbols():
    syms = declared_symbols()
    required = ["cubbs_bbs_gpu_sign_batch_v2", "cubbs_bbs_gpu_verify_batch_v2",
                "cubbs_bbs_gpu_proof_gen_batch_v2", "cubbs_bbs_gpu_proof_verify_batch_v2"]
    for r in required:
        assert r in syms
    assert len(syms) >= 23


def test_library_exports_all_declared_symbols():
    pkg = load_package()
    path = pkg.build()
    lib = ctypes.CDLL(str(path))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_abi_version_rejected_without_device_work():
    pkg = load_package()
    pkg.build()
    lib = pkg.lib()
    res = (pkg.Result * 1)()
    # a wrong ABI version is rejected before any CUDA call is made
    assert lib.cubbs_bbs_gpu_sign_batch_v2(1, None, 0, ctypes.cast(res, ctypes.c_void_p)) == pkg.ERR_INVALID_INPUT
    assert lib.cubbs_bbs_gpu_backend_info_v2(3, None) == pkg.ERR_INVALID_INPUT
    # null items with a nonzero count are malformed arguments
    assert lib.cubbs_bbs_gpu_verify_batch_v2(2, None, 4, ctypes.cast(res, ctypes.c_void_p)) == pkg.ERR_INVALID_INPUT


def test_no_oracle_in_product():
    """The product sources never reference the oracle."""
    for p in (ROOT / "cubbs-cred_gb300").rglob("*"):
        if p.suffix in (".cu", ".cuh", ".py", ".h", ".cpp") and "_build" not in p.parts:
            assert "oracle" not in p.read_text().lower(), p
