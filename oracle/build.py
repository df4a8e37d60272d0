"""Builds the CPU oracle (test infrastructure only) and, when the Voreen
sources are present, the reference pin library under ``oracle/_ref``.

liborc.so   : oracle/cpu_raycaster.cpp, g++ -O3 -fopenmp -ffp-contract=off.
_ref/libvoreen_ref.so : the reference's own VolumeRAM trilinear code
              (src/core/datastructures/volume/volumeram.cpp) plus the tgt
              header-only math, compiled from the reference tree with a link
              shim and a small driver (oracle/ref_pin/). Used only to make the
              golden vectors in tests/golden and to cross-check the oracle.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liborc.so")
REF_LIB = os.path.join(REF_OUT, "libvoreen_ref.so")
# The Voreen source tree (read only) for the reference pin library: taken from
# VOREEN_REFERENCE when set; absent on machines without the reference.
DEFAULT_REFERENCE = os.environ.get("VOREEN_REFERENCE", "/root/reference/voreen")


def _cxx() -> str:
    return os.environ.get("CXX") or shutil.which("g++") or "g++"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "cpu_raycaster.cpp")
    hdr = os.path.join(HERE, "oracle.h")
    if force or _stale(LIB, [src, hdr]):
        cmd = [_cxx(), "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return LIB


SYNTH_SRC = os.path.join(os.path.dirname(HERE), "voreen_gb300", "csrc", "synth.cpp")
SYNTH_LIB = os.path.join(BUILD, "libsynth.so")


def build_synth(force: bool = False) -> str:
    """The seeded workload generator (vrc_synth_volume) built on its own, so
    that the benchmark's CPU arm makes the same input volumes as the GPU arm
    without loading the product library."""
    os.makedirs(BUILD, exist_ok=True)
    hdr = os.path.join(os.path.dirname(HERE), "include", "vrc_synth.h")
    if force or _stale(SYNTH_LIB, [SYNTH_SRC, hdr]):
        cmd = [_cxx(), "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", SYNTH_SRC, "-o", SYNTH_LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"workload generator build failed:\n{r.stderr}")
    return SYNTH_LIB


def build_ref(reference_root: str = DEFAULT_REFERENCE, force: bool = False) -> str | None:
    """Compile the reference pin library; returns None when the reference
    tree is absent (it is not available everywhere)."""
    vr = os.path.join(reference_root, "src/core/datastructures/volume/volumeram.cpp")
    if not os.path.exists(vr):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    pin = os.path.join(HERE, "ref_pin")
    srcs = [vr, os.path.join(pin, "link_shim.cpp"), os.path.join(pin, "driver.cpp")]
    if not force and not _stale(REF_LIB, srcs[1:]) and os.path.exists(REF_LIB):
        return REF_LIB
    inc = []
    for d in ("", "ext", "include", "ext/boost/include", "ext/rapidjson", "ext/tinyxml", "ext/glew/include"):
        inc += ["-I", os.path.join(reference_root, d)]
    flags = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-DUNIX", "-DTIXML_USE_STL", "-w"]
    objs = []
    for s in srcs:
        o = os.path.join(REF_OUT, os.path.basename(s) + ".o")
        r = subprocess.run([_cxx(), *flags, *inc, "-c", s, "-o", o], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference pin build failed for {s}:\n{r.stderr[-4000:]}")
        objs.append(o)
    r = subprocess.run([_cxx(), "-shared", "-o", REF_LIB, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference pin link failed:\n{r.stderr[-4000:]}")
    return REF_LIB


REF_TF_LIB = os.path.join(REF_OUT, "libvoreen_tf_ref.so")


def build_tf_ref(reference_root: str = DEFAULT_REFERENCE, force: bool = False) -> str | None:
    """Compile the reference's own TF bake arithmetic into
    oracle/_ref/libvoreen_tf_ref.so: TransFunc1DKeys::getMappingForValueUByte
    (transfunc1dkeys.cpp), TransFunc1D::applyGammaToIntensity (transfunc1d.cpp)
    and TransFuncMappingKey (transfuncmappingkey.cpp), driven by
    oracle/ref_pin/tf_driver.cpp. Hidden visibility and section garbage
    collection keep only what the driver reaches, so the GL, shader and
    serialisation code those files also hold is dropped at link time.
    Returns None when the reference tree is absent."""
    base = os.path.join(reference_root, "src/core/datastructures/transfunc/1d")
    srcs = [os.path.join(base, "1dkeys/transfunc1dkeys.cpp"), os.path.join(base, "transfunc1d.cpp"),
            os.path.join(base, "1dkeys/utils/transfuncmappingkey.cpp"), os.path.join(HERE, "ref_pin", "tf_driver.cpp")]
    if not all(os.path.exists(s) for s in srcs):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    if not force and not _stale(REF_TF_LIB, srcs[3:]) and os.path.exists(REF_TF_LIB):
        return REF_TF_LIB
    inc = []
    for d in ("", "ext", "include", "ext/boost/include", "ext/rapidjson", "ext/tinyxml", "ext/glew/include"):
        inc += ["-I", os.path.join(reference_root, d)]
    flags = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-DUNIX", "-DTIXML_USE_STL",
             "-DBOOST_SYSTEM_NO_DEPRECATED", "-w", "-fvisibility=hidden", "-ffunction-sections", "-fdata-sections"]
    objs = []
    for s in srcs:
        o = os.path.join(REF_OUT, "tf_" + os.path.basename(s) + ".o")
        r = subprocess.run([_cxx(), *flags, *inc, "-c", s, "-o", o], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference TF pin build failed for {s}:\n{r.stderr[-4000:]}")
        objs.append(o)
    r = subprocess.run([_cxx(), "-shared", "-Wl,--gc-sections", "-o", REF_TF_LIB, *objs], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference TF pin link failed:\n{r.stderr[-4000:]}")
    return REF_TF_LIB


if __name__ == "__main__":
    print(build(force=True))
    print(build_ref(force=True))
    print(build_tf_ref(force=True))
