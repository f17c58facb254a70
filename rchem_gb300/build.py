"""Build librchem_gpu.so in-tree for sm_103a (GB300).

Steps: run the ERI code generator (csrc/gen_eri.py -> csrc/_gen/), compile
every translation unit with nvcc in parallel (one per ERI class plus the C-ABI
unit), link a shared library next to this file.  A stamp over the sources and
flags skips work that is already done.
"""
from __future__ import annotations

import hashlib
import importlib.util
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
GEN = os.path.join(CSRC, "_gen")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librchem_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librchem_gpu.so")


def _generate():
    spec = importlib.util.spec_from_file_location("rchem_gen_eri", os.path.join(CSRC, "gen_eri.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.main(GEN)


def _digest(paths, extra):
    h = hashlib.sha256()
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    h.update(repr(extra).encode())
    return h.hexdigest()


def ptxas_extra(src: str) -> list:
    """Extra nvcc flags of one translation unit: ptxas -O1 for the one-lane-group
    kernels of the classes of total angular momentum 6 and 7 (csrc/gen_eri.py
    SPLIT_L, generated as eri_<class>_cls.cu) and the FP64 (pp|pp) gradient
    kernel.  At -O1 ptxas keeps their values in registers (255 of them, 2-8 KB
    of local memory per thread) where -O3 gives the L = 6 ERI kernels 32
    registers and ~19 KB (twice as slow) and the gradient one ~30 KB, and takes
    minutes over the L = 7 one."""
    return ["-Xptxas", "-O1"] if src.endswith(("_cls.cu", "grad_pppp_f64.cu")) else []


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hand = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh", ".h", ".py"))]
    hand += [os.path.join(INCLUDE, f) for f in sorted(os.listdir(INCLUDE))]
    stamp = os.path.join(BUILD, "stamp")
    key = _digest(hand, (ARCH, NVFLAGS))
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == key:
        return LIB
    _generate()
    srcs = [os.path.join(CSRC, f) for f in ("rchem_gpu.cu", "peak.cu", "grad_sp_f64.cu", "grad_pppp_f64.cu", "grad_sp_f32.cu",
                                            "grad_sp_df64.cu", "grad_sp_df64b.cu", "grad_sd_f64.cu",
                                            "grad_sd_f32.cu", "onee_cls.cu")]
    srcs += sorted(os.path.join(GEN, f) for f in os.listdir(GEN) if f.startswith("eri_") and f.endswith(".cu"))
    nvcc = _nvcc()

    headers = [os.path.join(CSRC, f) for f in ("eri_kernel.cuh", "boys.cuh", "df64.cuh", "pq_table.cuh", "rchem_types.h")]

    def tag(src):  # the class of a generated translation unit (eri_<tag>.cu, eri_<tag>_cls.cu)
        return os.path.basename(src)[4:8]

    def deps(src):
        base = os.path.basename(src)
        if base.startswith("eri_") and src.startswith(GEN):
            prog = os.path.join(GEN, "eri_prog_%s.inc" % tag(src))
            return ([src, os.path.join(GEN, "eri_class_%s.inc" % tag(src))] +
                    ([prog] if os.path.exists(prog) else []) + headers)
        if base == "peak.cu":
            return [src, os.path.join(INCLUDE, "rchem_bench.h")]
        return [src] + hand + [os.path.join(GEN, "eri_dispatch.h"), os.path.join(GEN, "eri_classes.h")]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
        extra = ptxas_extra(src)
        okey = _digest(deps(src), (ARCH, NVFLAGS, extra, nvcc))
        hfile = obj + ".key"
        if not force and os.path.exists(obj) and os.path.exists(hfile) and open(hfile).read() == okey:
            return obj
        cmd = [nvcc, *ARCH, *NVFLAGS, *extra, "-I", CSRC, "-I", INCLUDE, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, r.stdout[-4000:], r.stderr[-8000:]))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        with open(hfile, "w") as f:
            f.write(okey)
        return obj

    # biggest classes first so the long compiles start early
    def class_size(s):
        inc = os.path.join(GEN, "eri_class_%s.inc" % tag(s))
        return os.path.getsize(inc) if s.startswith(GEN) and os.path.exists(inc) else 0

    srcs.sort(key=lambda s: -class_size(s))
    with ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout[-4000:], r.stderr[-8000:]))
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(key)
    return LIB


if __name__ == "__main__":
    import time

    t0 = time.time()
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print("%.1f s" % (time.time() - t0))
