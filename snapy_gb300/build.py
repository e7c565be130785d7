"""Build the in-tree CUDA library ``snapy_gb300/libsnapy_gb300.so`` (sm_103a).

The translation units below, compiled in parallel with nvcc and linked into one
shared library whose C ABI is ``include/snapy_gb300.h``:

* ``sg_stage.cu`` as FP64 with ``-fmad=false`` (the parity path: no
  contraction, the reference CPU path's rounding),
* ``sg_stage.cu`` as FP32 (contraction allowed),
* ``sg_api.cu`` (host bookkeeping and the small finishing kernels),
* ``sg_cs.cu`` as the cubed sphere's host API with its FP64 kernels
  (``-fmad=false``) and again as its FP32 kernels (contraction allowed).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsnapy_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required")


def _units():
    common = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-O3", "--expt-relaxed-constexpr"]
    stage = os.path.join(CSRC, "sg_stage.cu")
    units = [
        (stage, os.path.join(BUILD, "sg_stage_f64.o"),
         common + ["-DSG_REAL=double", "-fmad=false"]),
        (stage, os.path.join(BUILD, "sg_stage_f32.o"),
         common + ["-DSG_REAL=float", "-DSG_REAL_IS_FLOAT"]),
    ]
    # every other translation unit once, FP64 parity rules (no contraction)
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") and f != "sg_stage.cu":
            units.append((os.path.join(CSRC, f),
                          os.path.join(BUILD, f[:-3] + ".o"),
                          common + ["-fmad=false"]))
    # the cubed sphere's FP32 kernels again, contraction allowed
    units.append((os.path.join(CSRC, "sg_cs.cu"),
                  os.path.join(BUILD, "sg_cs_f32.o"),
                  common + ["-DSG_CS_F32_UNIT"]))
    return units


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "snapy_gb300.h"), __file__]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def compile_one(unit):
        src, obj, flags = unit
        cmd = [nv, "-c", src, "-o", obj] + list(flags) + list(extra_flags)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}{r.stderr}")
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        objs = list(ex.map(compile_one, _units()))
    tmp = LIB + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv,
          extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else [])
    print(LIB)
