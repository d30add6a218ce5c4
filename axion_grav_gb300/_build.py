"""Build recipe of libaxgpu.so (CUDA, sm_103a) -- compiled in-tree with nvcc.

Every translation unit under csrc/ is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo`` and linked into
``axion_grav_gb300/libaxgpu.so`` against cuFFT.  Host code is compiled with
``-ffp-contract=off`` so host-computed kick coefficients are bit-identical on
x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libaxgpu.so")
ROOT = os.path.dirname(PKG)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_lib_dir(nvcc: str) -> str:
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for sub in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"),
                os.path.join("targets", "x86_64-linux", "lib")):
        d = os.path.join(root, sub)
        if os.path.exists(os.path.join(d, "libcufft.so")):
            return d
    return os.path.join(root, "lib64")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


# Translation units whose device arithmetic must round every operation
# separately (no FMA contraction) so results are bit-identical to IEEE host C.
FMAD_OFF = {"axg_defects.cu"}


def _compile(nvcc: str, src: str, verbose_ptxas: bool) -> tuple[str, str]:
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    if os.path.basename(src) in FMAD_OFF:
        cmd.append("-fmad=false")
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile csrc/*.cu for sm_103a and link libaxgpu.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(ROOT, "include", "axgpu.h"))
    deps = srcs + headers + [os.path.abspath(__file__)]
    if not force and not verbose_ptxas and not _stale(LIB, deps):
        return LIB
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, verbose_ptxas), srcs))
    objs = [o for o, _ in results]
    if verbose_ptxas:
        for _, log in results:
            sys.stderr.write(log)
    libdir = _cuda_lib_dir(nvcc)
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-L" + libdir, "-lcufft",
           "-Xlinker", "-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
