"""The C-ABI library loads and exports every symbol include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(vrcp?_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(vrc_lib):
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(vrc_lib, n)]
    assert not missing, missing


def test_python_signatures_cover_the_headers(vrc_lib):
    from voreen_gb300 import _abi
    assert declared_symbols() == set(_abi.SIGNATURES) | set(_abi.NN_SIGNATURES) | set(_abi.PROC_SIGNATURES)


def test_host_only_entry_points_work_without_gpu(vrc_lib):
    assert vrc_lib.vrc_abi_version() == 2
    assert vrc_lib.vrc_status_string(0) == b"ok"
    assert vrc_lib.vrc_tf_table_width(0) == 256
    assert vrc_lib.vrc_tf_table_width(1) == 4096
    assert vrc_lib.vrc_tf_table_width(2) == 4096
