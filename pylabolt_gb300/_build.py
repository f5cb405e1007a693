"""Build recipe for liblbm_gb300.so (in-tree, sm_103a only).

Each translation unit is compiled by nvcc in parallel (one per storage type,
the FP32 / FP16 fused step split by collision model, the shared helpers, the
C-ABI and the allocation-free entry); the FP64 unit gets
``--fmad=false`` so that it keeps the reference's rounding.  The result is
``pylabolt_gb300/_build/liblbm_gb300.so`` (git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "liblbm_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-I", INCLUDE, "-I", CSRC]
UNITS = {
    "lbm_fp64.cu": ["--fmad=false"],
    "lbm_fp32.cu": [],
    "lbm_fp32_bgk.cu": [],
    "lbm_fp32_mrt.cu": [],
    "lbm_fp16.cu": [],
    "lbm_fp16_bgk.cu": [],
    "lbm_fp16_mrt.cu": [],
    "lbm_lowp.cu": [],
    "lbm_capi.cu": [],
    "lbm_noalloc.cu": [],
}


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")


def _sources_newest():
    newest = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            newest = max(newest, os.path.getmtime(os.path.join(d, f)))
    return max(newest, os.path.getmtime(__file__))


def build(force=False, verbose=False, extra_flags=()):
    """Compile (if stale) and return the path of liblbm_gb300.so."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_newest():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()

    def compile_unit(item):
        name, flags = item
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        cmd = [exe, *ARCH, *COMMON, *flags, *extra_flags, "-c",
               os.path.join(CSRC, name), "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS.items()))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
