"""The ctypes mirrors of the C ABI's structs (gbhsolve/engine.py,
gbhsolve/hsolve.py) have the layout include/gbhsolve.h and
include/gbh_hsolve.h give them: the same size and every field at the
same offset, as a C compiler lays them out on this host. A field added on one
side only would make the library read or write past the caller's struct."""
import ctypes as C
import re
import shutil
import subprocess

import pytest

from gbhsolve import build, engine, hsolve

STRUCTS = [("gbh_error", engine.GbhError), ("gbh_tables", engine.GbhTables),
           ("gbh_batch_desc", engine.GbhBatchDesc), ("gbh_synapses", engine.GbhSynapses),
           ("gbh_remote_synapses", engine.GbhRemoteSynapses), ("gbh_options", engine.GbhOptions),
           ("gbh_loss_spec", engine.GbhLossSpec), ("gbh_stats", engine.GbhStats),
           # the hsolve-level ABI (include/gbh_hsolve.h, gbhsolve/hsolve.py)
           ("gbh_hs_input", hsolve.HsInput), ("gbh_hs_synapse", hsolve.HsSynapse),
           ("gbh_hs_solver", hsolve.HsSolver)]


def _c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "gbh_hsolve.h"', "int main(void) {"]
    for cname, cls in STRUCTS:
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in cls._fields_:
            if fname.startswith("_"):
                continue
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    exe = tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-I", build.INCLUDE, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        m = re.match(r"(\w+) (\w+) (\d+)$", line)
        layout[(m.group(1), m.group(2))] = int(m.group(3))
    return layout


def test_ctypes_structs_match_the_header(tmp_path):
    layout = _c_layout(tmp_path)
    for cname, cls in STRUCTS:
        assert C.sizeof(cls) == layout[(cname, "size")], cname
        for fname, _ in cls._fields_:
            if fname.startswith("_"):
                continue
            assert getattr(cls, fname).offset == layout[(cname, fname)], (cname, fname)
