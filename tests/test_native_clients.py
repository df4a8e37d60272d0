"""The C ABI and the processor shim from native code: a C99 program and a
C++ program compiled against include/*.h with the host compilers and linked
to libvrc.so, running their host-only checks (no GPU)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "voreen_gb300", "_build")


def _build_and_run(tmp_path, src, compiler, std, args=()):
    cc = shutil.which(compiler)
    if cc is None:
        pytest.skip(f"{compiler} not found")
    exe = str(tmp_path / os.path.splitext(os.path.basename(src))[0])
    cmd = [cc, std, "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "native", src),
           "-L", LIBDIR, "-lvrc", f"-Wl,-rpath,{LIBDIR}", "-lm", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr + r.stdout
    return r.stdout


def test_c99_client(vrc_lib, tmp_path):
    tfi = tmp_path / "t.tfi"
    tfi.write_text('<VoreenData><TransFuncIntensity><Keys><key><intensity value="0.5" /><split value="false" />'
                   '<colorL r="1" g="2" b="3" a="4" /></key></Keys></TransFuncIntensity></VoreenData>')
    assert "abi_c99 ok" in _build_and_run(tmp_path, "abi_c99.c", "gcc", "-std=c99", [str(tfi)])


def test_cpp_processor_client(vrc_lib, tmp_path):
    assert "processor_cpp ok" in _build_and_run(tmp_path, "processor_cpp.cpp", "g++", "-std=c++17")
