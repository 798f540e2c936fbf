"""Build the solver library in-tree: ``libcupdlpx_gb300.so`` next to this file.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into
one shared library with the CUDA runtime linked statically, so the library
depends on nothing but the driver.  Re-running only recompiles sources newer
than their objects.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcupdlpx_gb300.so")

SOURCES = ["solver.cu", "solver_f32.cu", "solver_mix.cu", "refine.cu", "precond.cu", "hooks.cu",
           "noalloc.cu", "memory.cu", "transpose.cu",
           "api.cpp", "serve.cpp", "lpgen.cpp", "mps.cpp", "wire.cpp"]
CLI = os.path.join(HERE, "cupdlpx")
# gzip-compressed MPS input where the zlib header and library exist
HAVE_ZLIB = os.path.exists("/usr/include/zlib.h")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(src: str) -> list[str]:
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
         "-I" + os.path.join(ROOT, "include"), "-I" + CSRC] + ARCH
    # extra nvcc flags for tuning builds (e.g. -DPDLP_PIPE_CTAS=3); objects
    # are rebuilt when they change
    f += os.environ.get("PDLP_NVCC_FLAGS", "").split()
    if src == "lpgen.cpp":
        f += ["-Xcompiler", "-ffp-contract=off"]  # bit-identical on x86 and Arm
    if src.endswith(".cu") or src in ("api.cpp", "serve.cpp"):
        f += ["--expt-relaxed-constexpr"]
    if src in ("api.cpp", "serve.cpp"):
        f = ["-x", "cu"] + f  # includes the device-side solver header
    if src == "mps.cpp" and HAVE_ZLIB:
        f += ["-DPDLP_HAVE_ZLIB"]
    return f


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    hs += [os.path.join(ROOT, "include", h) for h in os.listdir(os.path.join(ROOT, "include"))]
    return max(os.path.getmtime(h) for h in hs)


def _compile(src: str, hdr_time: float) -> str:
    out = os.path.join(OBJ, src + ".o")
    path = os.path.join(CSRC, src)
    stamp = out + ".flags"
    flags = " ".join(_flags(src))
    same_flags = os.path.exists(stamp) and open(stamp).read() == flags
    if same_flags and os.path.exists(out) and \
            os.path.getmtime(out) >= max(os.path.getmtime(path), hdr_time):
        return out
    cmd = [nvcc(), "-c", path, "-o", out] + _flags(src)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as fh:
        fh.write(flags)
    return out


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    hdr = _headers_mtime()
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr), SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-cudart", "static"] + \
            (["-lz"] if HAVE_ZLIB else [])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    src = os.path.join(CSRC, "cli.cpp")
    if not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(LIB),
                                                              os.path.getmtime(src), hdr):
        # the command-line tool, linked against the library beside it
        cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
               src, "-o", CLI, "-L" + HERE, "-lcupdlpx_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
