"""Builds the in-tree CUDA library ``voreen_gb300/_build/libvrc.so`` for sm_103a.

Every translation unit is compiled by nvcc in parallel and linked into one
shared library exporting the C ABI of ``include/vrc.h`` (plus
``include/vrc_synth.h``). Nothing is installed outside the tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libvrc.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off", "-I", INCLUDE,
          "-I", CSRC]
# The march path rounds every operation explicitly; -fmad=false keeps any
# remaining plain arithmetic on that path from being fused as well.
SOURCES = [
    ("api.cpp", []),
    ("synth.cpp", []),
    ("volume.cu", []),
    ("march.cu", ["-fmad=false"]),
    ("march_dvr.cu", ["-fmad=false"]),
    ("march_mip_iso.cu", ["-fmad=false"]),
    ("march_mop_mida.cu", ["-fmad=false"]),
    ("march_first_hit.cu", ["-fmad=false"]),
    ("preint.cu", ["-fmad=false"]),
    ("image.cu", []),
    ("diag.cu", []),
    ("ingest.cpp", []),
    ("noalloc.cu", []),
    ("batch.cpp", []),
    ("processor.cpp", []),
    ("nn.cu", []),
    ("nn_tc.cu", []),
    ("synth_tubes.cu", []),
]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build voreen_gb300")
    return cand


def _headers() -> list[str]:
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile and link libvrc.so. Environment tuning knobs:
    VRC_MARCH_MIN_BLOCKS (march kernels: minimum resident CTAs per SM, bounds
    the registers; default 3), VRC_OCC_DIST_CAP (largest empty-space distance
    stored per cell, at most 255; default 16) and VRC_CELL2_LOG2_MAX (the 2^3
    cell level is built for volumes of at most 2^this cells; default 30).
    Objects are rebuilt when their knobs differ from the last build's."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    stamps = []
    for src, extra in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace(".", "_") + ".o")
        objs.append(obj)
        tune = [f"-D{k}={int(os.environ[k])}" for k in ("VRC_MARCH_MIN_BLOCKS",)
                if src.startswith("march") and os.environ.get(k)]
        tune += [f"-DVRC_OCC_DIST_CAP={int(os.environ['VRC_OCC_DIST_CAP'])}"] if os.environ.get("VRC_OCC_DIST_CAP") else []
        tune += [f"-DVRC_CELL2_LOG2_MAX={int(os.environ['VRC_CELL2_LOG2_MAX'])}"] if os.environ.get("VRC_CELL2_LOG2_MAX") else []
        extra = extra + tune
        # an object is rebuilt when its tuning flags differ from the last build's
        stamp = obj + ".flags"
        flags = " ".join(tune)
        force_this = (open(stamp).read() if os.path.exists(stamp) else "") != flags
        if force or force_this or _stale(obj, [path] + hdrs):
            stamps.append((stamp, flags))
            cmd = [cc, *ARCH, *COMMON, *extra, "-c", path, "-o", obj]
            if src.endswith(".cpp"):
                cmd.insert(1, "-x")
                cmd.insert(2, "cu")
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err)
    for stamp, flags in stamps:
        with open(stamp, "w") as f:
            f.write(flags)
    if force or jobs or _stale(LIB, objs):
        run([cc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
