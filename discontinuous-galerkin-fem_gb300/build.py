"""Build ``libdgx.so`` (the C-ABI library of include/dgx.h) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into one shared
library next to this file.  Usage:  python build.py [--force] [--verbose]
"""

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "libdgx.so"
OBJ = HERE / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["dgx_host.cpp", "dgx_kernels_fp64.cu", "dgx_kernels_mixed.cu", "dgx_misc.cu", "dgx_static.cu", "dgx_adjoint.cu",
           "dgx_batch.cu", "dgx_batch_host.cpp", "dgx_tune.cpp", "dgx_kernels_tc.cu",
           "dgx_kernels_df64.cu", "dgx_quad.cu", "dgx_kernels_trace.cu", "dgx_kernels_trace_small.cu", "dgx_kernels_trace_nbs.cu",
           "dgx_setup.cu"]
HEADERS = ["dgx_internal.h", "dgx_context.h", "dg_physics.cuh", "dg_element.cuh", "dg_stage.cuh", "dg_adjoint.cuh", "dg_stage_tc.cuh", "tc_ptx.cuh", "df64.cuh", "dg_quad.cuh", "dg_stage_trace.cuh", "fp_bits.cuh", "quad_tables.inc"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _flags():
    # host code without floating-point contraction: the set-up arithmetic then rounds the same on
    # every host CPU and equals the device set-up's (dgx_setup.cu)
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
                   "-I", str(HERE.parent / "include")]


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force=False, verbose=False) -> Path:
    OBJ.mkdir(exist_ok=True)
    nv = nvcc()
    hdrs = [CSRC / h for h in HEADERS] + [HERE.parent / "include" / "dgx.h", Path(__file__)]
    jobs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = OBJ / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [nv] + _flags() + ["-c", str(s), "-o", str(o)]
            if s.suffix == ".cpp":
                cmd[1:1] = ["-x", "cu"]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"nvcc failed: {cmd[-3]}")
    if force or jobs or _stale(OUT, objs):
        cmd = [nv] + ARCH + ["-shared", "-o", str(OUT)] + [str(o) for o in objs] + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.verbose))
