"""The GENESIS-side adapter (genesis-2.4_gb300/adapter/gbh_hsolve_adapter.c)
compiles against the reference's own headers (hines_ext.h, hines_struct.h)
with the reference's compiler flags, and every engine symbol it calls is
exported by libgbhsolve.so."""
import os
import re
import subprocess

import pytest

from gbhsolve import build

import pyoracle

REF = pyoracle.reference_src()
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(REPO, "genesis-2.4_gb300", "adapter", "gbh_hsolve_adapter.c")


@pytest.mark.skipif(not REF or not os.path.exists(REF + "/hines/hines_ext.h"), reason="reference headers not present")
def test_adapter_compiles_against_reference_headers(tmp_path):
    inc = sum((["-I", REF + "/" + d] for d in ("hines", "sim", "ss", "shell", "segment", "olf", "concen",
                                                 "device", "newconn", "sys")), [])
    obj = tmp_path / "adapter.o"
    r = subprocess.run(["gcc", "-c", "-O2", "-DLONGWORDS", "-std=gnu99", "-Wall", "-Wno-unused-variable",
                        "-I", os.path.join(REPO, "include")] + inc + [ADAPTER, "-o", str(obj)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    undef = subprocess.run(["nm", "-u", str(obj)], capture_output=True, text=True).stdout
    calls = set(re.findall(r"\b(gbh_[a-z_]+)\b", undef))
    lib = build.build()
    exported = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    for name in calls:
        assert re.search(r"\bT %s\b" % name, exported), name
