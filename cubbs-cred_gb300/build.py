"""Build libcubbs_bbs_cuda.so (sm_103a) in-tree.

Each translation unit under csrc/ is compiled by nvcc in parallel, then linked
into cubbs-cred_gb300/lib/libcubbs_bbs_cuda.so.  Objects go to _build/.
Rebuilds only what changed (source or any header newer than the object).
"""
import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parent
CSRC = ROOT / "csrc"
BUILD = ROOT / "_build"
LIBDIR = ROOT / "lib"
LIB = LIBDIR / "libcubbs_bbs_cuda.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = ["runtime", "k_hash", "k_g1", "k_pairing", "k_bbs", "k_prims", "k_selftest", "k_noalloc", "serve", "k_msm", "proofvalue", "bbs2023"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + list((ROOT.parent / "include").glob("*.h"))
    return max(h.stat().st_mtime for h in hs)


def _compile(unit: str, nvcc: str, hdr_mtime: float, verbose: bool) -> pathlib.Path:
    src = CSRC / f"{unit}.cu"
    obj = BUILD / f"{unit}.o"
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_mtime):
        return obj
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    (BUILD / f"{unit}.log").write_text(res.stdout + res.stderr)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{res.stderr[-4000:]}")
    return obj


def build(verbose: bool = False) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    nvcc = _nvcc()
    hdr = _headers_mtime()
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u, nvcc, hdr, verbose), UNITS))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB
    cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr[-4000:]}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
