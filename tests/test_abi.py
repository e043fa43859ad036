"""CPU: the C-ABI library builds, loads without a GPU, and exports every
function include/gbglioma.h declares. No compute calls."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "gbglioma.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbg_[a-z0-9_]+)\s*\(", text)))


def test_header_lists_expected_entry_points():
    names = declared_functions()
    from gliomauq_gb300 import _lib
    assert set(names) == set(_lib.EXPORTS), (set(names) ^ set(_lib.EXPORTS))


def test_library_exports_every_declared_symbol(gbg):
    for name in declared_functions():
        assert hasattr(gbg, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", gbg._name], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (gbg_\w+)", out))
    assert set(declared_functions()) <= exported


def test_version_and_error_without_gpu_compute(gbg):
    import ctypes as C
    ma, mi = C.c_int(), C.c_int()
    assert gbg.gbg_version(C.byref(ma), C.byref(mi)) == 0
    assert (ma.value, mi.value) == (0, 1)
    # a null config is rejected before any CUDA call
    assert gbg.gbg_create(None, None) == -1
    assert b"null" in gbg.gbg_last_error()
