"""Builds libc2a_gb300.so in-tree for sm_103a (GB300).

Device code: nvcc, ``-gencode arch=compute_103a,code=sm_103a``, ``--fmad=false``
(every FP64 product and sum rounds on its own, as in the reference's x86
build).  Host code: g++ through nvcc with ``-ffp-contract=off``.  The CUDA
runtime is linked statically, so the library loads on a machine without a GPU
(its query entry points then report ``C2A_ERR_NO_DEVICE``).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libc2a_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["c2a_abi.cu", "k_thread.cu", "k_warp.cu", "k_spec.cu", "k_front.cu", "k_static.cu", "c2a_wave.cu", "mlp.cu", "probe.cu"]
HOST_SOURCES = ["host/bvh_build.cpp", "host/c2a_api.cpp"]
HOST_FLAGS = "-fPIC,-O2,-ffp-contract=off,-fno-fast-math,-Wall"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _sources() -> list[str]:
    out = []
    for root, _, files in os.walk(CSRC):
        out += [os.path.join(root, f) for f in files]
    out.append(os.path.join(HERE, "..", "include", "c2a_gb300.h"))
    out.append(os.path.join(HERE, "..", "include", "c2a_gb300_cpp.h"))
    out.append(os.path.join(HERE, "..", "include", "c2a_mlp.h"))
    return [p for p in out if os.path.exists(p)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False, defines: tuple = (),
          lib: str = LIB) -> str:
    """Compiles every translation unit in parallel and links the shared library.

    ``defines`` (e.g. ``("C2A_STATS",)`` for the event-counting profiling
    build) and ``lib`` make a variant library elsewhere; the default is the
    product library.
    """
    if not force and lib == LIB and not defines and up_to_date():
        return LIB
    out_dir = os.path.dirname(os.path.abspath(lib))
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    dflags = [f"-D{d}" for d in defines]
    jobs = []
    for src in CUDA_SOURCES:
        obj = os.path.join(out_dir, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "--fmad=false", "-std=c++17", *dflags, "-Xcompiler", HOST_FLAGS,
               "-c", os.path.join(CSRC, src), "-o", obj]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((cmd, obj))
    for src in HOST_SOURCES:
        obj = os.path.join(out_dir, os.path.basename(src) + ".o")
        cmd = [nvcc, "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", HOST_FLAGS, "-c", os.path.join(CSRC, src),
               "-o", obj]
        jobs.append((cmd, obj))

    def run(job):
        cmd, _ = job
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(run, jobs))
    if ptxas_info:
        print("\n".join(logs), file=sys.stderr)
    tmp = lib + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp] + [o for _, o in jobs]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
