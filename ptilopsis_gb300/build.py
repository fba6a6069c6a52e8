"""In-tree build of the package's native libraries.

  ptilopsis_gb300/_lib/libptl_gb300.so      CUDA code generator (sm_103a), C ABI of
                                            include/ptl_codegen.h
  ptilopsis_gb300/_lib/libptlsynth.so       seeded synthetic program generator
  ptilopsis_gb300/_lib/libptl_hostmodel.so  test-only CPU build of the GPU stage logic

nvcc and g++ run directly (no cmake); translation units compile in parallel.  Builds
are skipped when every output is newer than every source.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter"]

CUDA_LIB = os.path.join(LIBDIR, "libptl_gb300.so")
SYNTH_LIB = os.path.join(LIBDIR, "libptlsynth.so")
HOSTMODEL_LIB = os.path.join(LIBDIR, "libptl_hostmodel.so")

HEADERS = ["ptl_device.h", "ptl_common.cuh", "ptl_stages.cuh", "ptl_sort.cuh", "ptl_ra.cuh", "ptl_scalar.cuh", "ptl_kernels.cuh",
           "ptl_bpipe.h"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 code generator needs the CUDA toolkit to build")


def _newer(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _src(*names: str) -> list[str]:
    return [os.path.join(CSRC, n) for n in names]


def build_cuda(force: bool = False) -> str:
    hdrs = _src(*HEADERS) + [os.path.join(ROOT, "include", "ptl_codegen.h")]
    units = [("ptl_kernels.cu", "nvcc"), ("ptl_capi.cu", "nvcc"), ("ptl_noalloc.cu", "nvcc"), ("ptl_bpipe.cu", "nvcc"),
             ("ptl_flatten.cu", "nvcc"), ("ptl_tables.cpp", "cxx"), ("ptl_batch.cpp", "cxx"), ("ptl_disasm.cpp", "cxx"), ("ptl_elf.cpp", "cxx")]
    all_src = _src(*(u for u, _ in units)) + hdrs
    if not force and _newer(CUDA_LIB, all_src):
        return CUDA_LIB
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for unit, tool in units:
        obj = os.path.join(OBJDIR, unit + ".o")
        if tool == "nvcc":
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, unit), "-o", obj]
        else:
            cmd = ["g++", *CXX_FLAGS, "-c", os.path.join(CSRC, unit), "-o", obj]
        jobs.append((cmd, obj))
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for f in [ex.submit(_run, cmd) for cmd, _ in jobs]:
            f.result()
    _run([nvcc, *ARCH, "-shared", "-o", CUDA_LIB, *[o for _, o in jobs], "-lcudart", "-lpthread"])
    return CUDA_LIB


def build_synth(force: bool = False) -> str:
    srcs = [os.path.join(CSRC, "synth", "ptl_synth.cpp"), os.path.join(CSRC, "synth", "ptl_synth.h")]
    if not force and _newer(SYNTH_LIB, srcs):
        return SYNTH_LIB
    os.makedirs(LIBDIR, exist_ok=True)
    _run(["g++", *CXX_FLAGS, "-ffp-contract=off", "-shared", "-o", SYNTH_LIB, srcs[0]])
    return SYNTH_LIB


def build_hostmodel(force: bool = False) -> str:
    srcs = _src("ptl_hostmodel.cpp", "ptl_tables.cpp", "ptl_common.cuh", "ptl_stages.cuh", "ptl_sort.cuh", "ptl_ra.cuh",
                "ptl_scalar.cuh")
    if not force and _newer(HOSTMODEL_LIB, srcs):
        return HOSTMODEL_LIB
    os.makedirs(LIBDIR, exist_ok=True)
    _run(["g++", *CXX_FLAGS, "-shared", "-o", HOSTMODEL_LIB, srcs[0], srcs[1]])
    return HOSTMODEL_LIB


def build_all(force: bool = False, cuda: bool = True) -> dict:
    out = {}
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = {"synth": ex.submit(build_synth, force), "hostmodel": ex.submit(build_hostmodel, force)}
        if cuda:
            futs["cuda"] = ex.submit(build_cuda, force)
        for k, f in futs.items():
            out[k] = f.result()
    return out


if __name__ == "__main__":
    print(build_all(force=True))
