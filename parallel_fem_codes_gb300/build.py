"""Compile libfemgpu (sm_103a) in-tree: parallel_fem_codes_gb300/_lib/libfemgpu.so.

One nvcc invocation per translation unit, run in parallel, then one link.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libfemgpu.so")
COMPAT_SST = os.path.join(OUT, "libfemgpu_sst.so")
COMPAT_NS = os.path.join(OUT, "libfemgpu_ns.so")
COMPAT_EULER = os.path.join(OUT, "libfemgpu_euler.so")
COMPAT_TT = os.path.join(OUT, "libfemgpu_tt.so")
COMPAT = [COMPAT_SST, COMPAT_NS, COMPAT_EULER, COMPAT_TT]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags); setup.cu is rounded exactly as written (no FMA
# contraction) so assembly and preconditioner set-up match the reference.
UNITS = [
    ("topology.cpp", []),
    ("meshio.cpp", []),
    ("system.cu", []),
    ("krylov.cu", []),
    ("setup.cu", ["-fmad=false"]),
    ("noalloc.cu", []),
    ("server.cu", []),
    ("ilu.cu", ["-fmad=false"]),
    ("spike.cu", ["-fmad=false"]),
    ("ns.cu", ["-fmad=false"]),
    ("euler.cu", ["-fmad=false"]),
]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT, "obj", os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
           "--expt-relaxed-constexpr", "-c", path, "-o", obj, *extra]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    subprocess.run(cmd, check=True)
    return obj


def build(force: bool = False) -> str:
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s, _ in UNITS]
    hdrs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    hdrs.append(os.path.join(os.path.dirname(PKG), "include", "femgpu.h"))
    srcs += [os.path.join(PKG, "compat", f) for f in os.listdir(os.path.join(PKG, "compat"))]
    if not force and all(os.path.exists(f) for f in [LIB] + COMPAT):
        t = min(os.path.getmtime(f) for f in [LIB] + COMPAT)
        if all(os.path.getmtime(f) < t for f in srcs + hdrs + [__file__]):
            return LIB
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), UNITS))
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"], check=True)
    # drop-in shims with the reference's entry-point names: steady transport,
    # steady Navier-Stokes, Euler and transient transport drivers (one per
    # struct layout)
    cc = os.environ.get("CC", "gcc")
    shims = [(COMPAT_SST, "compat_sst.c", []), (COMPAT_NS, "compat_block.c", ["-DFGC_NS"]),
             (COMPAT_EULER, "compat_block.c", ["-DFGC_EULER"]), (COMPAT_TT, "compat_sst.c", ["-DFGC_TT"])]
    for out, src, defs in shims:
        subprocess.run([cc, "-O2", "-fPIC", "-shared", "-std=gnu99", "-Wall", *defs, "-o", out,
                        os.path.join(PKG, "compat", src), "-L" + OUT, "-lfemgpu", "-Wl,-rpath,$ORIGIN"],
                       check=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
