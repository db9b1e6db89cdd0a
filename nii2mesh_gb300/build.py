"""Build recipe for libn2m_gpu.so (sm_103a) — invoked by __graft_entry__.build().

Every translation unit in csrc/ is compiled in parallel with nvcc for
sm_103a only (no PTX fallback, no other architectures), then linked into one
shared library with a C ABI (include/n2m_gpu.h).  Floating-point contraction
is disabled (--fmad=false) because several stages must reproduce the
reference's IEEE operation sequence bit for bit; divisions and square roots
stay IEEE-rounded (no fast math).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libn2m_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
         "-I", str(CSRC), "-I", str(PKG.parent / "include")]
# units with bit-exact floating-point duties: smoothing, marching cubes (both
# builds), the weld and degenerate filter, sform, Otsu, the NIfTI cast, the
# batched atlas, the text writers and the host-side glue
EXACT = {"smooth", "mc", "oldcubes", "mesh", "isolevel", "decode", "atlas", "writers", "capi"}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(CSRC.glob("*.cu"))


def build(verbose=False, force=False, extra=()):
    OUT.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    deps = srcs + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [PKG.parent / "include" / "n2m_gpu.h"]
    if LIB.exists() and not force and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    cc = nvcc()

    def compile_one(src):
        obj = OUT / (src.stem + ".o")
        fmad = ["--fmad=false"] if src.stem in EXACT else []
        cmd = [cc, *ARCH, *FLAGS, *fmad, *extra, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv,
                extra=("-Xptxas", "-v") if "--ptxas" in sys.argv else ()))
