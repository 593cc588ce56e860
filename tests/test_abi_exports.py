"""The C-ABI library builds, loads without a GPU, and exports every function
declared in include/*.h (gbhsolve.h: the array-level ABI; gbh_hsolve.h: the
hsolve-level ABI)."""
import ctypes
import os
import re

from gbhsolve import build, engine

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(REPO, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(gbh_[a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("gbh_create", "gbh_run", "gbh_get_state", "gbh_destroy", "gbh_validate",
                     "gbh_run_noalloc", "gbh_hs_register", "gbh_hs_step", "gbh_hs_sync", "gbh_hs_push"):
        assert required in names


def test_library_loads_and_exports_every_declared_symbol():
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert sorted(engine.EXPORTED) == declared_functions()


def test_step_entry_points_reject_a_null_engine_before_any_device_call():
    """A NULL engine or a negative step count is GBH_ERR_ARG, decided on the
    host before any CUDA call, so it holds on a machine without a GPU."""
    lib = ctypes.CDLL(build.build())
    GBH_ERR_ARG = -1
    for name in ("gbh_run", "gbh_run_noalloc", "gbh_step_io", "gbh_run_io"):
        getattr(lib, name).restype = ctypes.c_int
    assert lib.gbh_run(None, 1) == GBH_ERR_ARG
    assert lib.gbh_run_noalloc(None, 1, None) == GBH_ERR_ARG
    assert lib.gbh_run_noalloc(None, -1, None) == GBH_ERR_ARG
    assert lib.gbh_step_io(None, None, None, 1, None) == GBH_ERR_ARG
    assert lib.gbh_run_io(None, None, None, 1, 16, None) == GBH_ERR_ARG
