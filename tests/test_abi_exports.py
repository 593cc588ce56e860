"""The C-ABI library builds, loads without a GPU, and exports every function
declared in include/gbhsolve.h."""
import ctypes
import os
import re

from gbhsolve import build, engine

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(REPO, "include", "gbhsolve.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(gbh_[a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("gbh_create", "gbh_run", "gbh_get_state", "gbh_destroy", "gbh_validate",
                     "gbh_run_noalloc"):
        assert required in names


def test_library_loads_and_exports_every_declared_symbol():
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert sorted(engine.EXPORTED) == declared_functions()
