"""The GENESIS adapter (genesis-2.4_gb300/adapter/gbh_hsolve_adapter.c) run as
GENESIS runs it: compiled against the reference's own headers together with
a minimal GENESIS host (tests/genesis_host/adapter_host.c) that builds each
Hsolve around an oracle solver's arrays, feeds INJECT messages through
MSGVALUE and steps PROCESS through gbh_init / gbh_chip_update, with
gbh_sync_chip and gbh_push_state for a RESTORE2-style edit in mid-run.

24 per-cell hsolves (random trees with Ca pools, backward Euler and
Crank-Nicolson mixed in one batch) are stepped 200 steps; every step the
scheduler calls all 24, the first call runs the batch. Vm of the solvers with
output messages is compared after every step, and all arrays at the end, bit
for bit with the reference's own step code (hines_4chip.c, hines_conc*.c,
hines_solve.c) given the same injects.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import pyoracle
from gbhsolve import build, configs, model

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(REPO, "genesis-2.4_gb300", "adapter", "gbh_hsolve_adapter.c")
HOST = os.path.join(REPO, "tests", "genesis_host", "adapter_host.c")
REF_DIRS = ("hines", "sim", "ss", "shell", "segment", "olf", "concen", "device", "newconn", "sys")


def _host_lib(tmp_path):
    ref = pyoracle.reference_src()
    if not pyoracle.reference_sources_present():
        pytest.skip("reference headers and step code not present")
    lib = build.build()
    libdir = os.path.dirname(lib)
    out = str(tmp_path / "libadapter_host.so")
    inc = sum((["-I", os.path.join(ref, d)] for d in REF_DIRS), [])
    cmd = (["gcc", "-shared", "-fPIC", "-O2", "-DLONGWORDS", "-std=gnu99", "-Wall", "-Wno-unused-variable",
            "-Wno-comment", "-I", os.path.join(REPO, "include"), "-I", os.path.join(REPO, "oracle")] + inc +
           [ADAPTER, HOST, "-L", libdir, "-lgbhsolve", "-Wl,-rpath," + libdir, "-o", out])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    h = C.CDLL(out)
    h.ah_create.restype = C.c_void_p
    h.ah_create.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
    for f in ("ah_init", "ah_push"):
        getattr(h, f).argtypes = [C.c_void_p]
    h.ah_process.argtypes = [C.c_void_p, C.c_double]
    h.ah_sync.argtypes = [C.c_void_p]
    h.ah_destroy_all.argtypes = [C.c_void_p, C.c_int]
    return h


def test_adapter_host_builds_and_loads(tmp_path):
    """The adapter and the host link against libgbhsolve.so and load (no GPU
    needed; nothing is stepped)."""
    host = _host_lib(tmp_path)
    assert host.ah_create and host.ah_process


@pytest.mark.gpu
def test_adapter_batch_equals_reference_step_code(tmp_path, oracle, gpu_engine):
    host = _host_lib(tmp_path)
    n, nsteps = 24, 200
    hs = [model.build(m) for m in configs.random_trees(n, size_range=(8, 64), seed=31, method=model.BEULER)]
    hs[1::3] = [model.build(m) for m in configs.random_trees(n, size_range=(8, 64), seed=32,
                                                               method=model.CRANK)][1::3]
    rng = np.random.default_rng(33)
    inj = rng.uniform(0.0, 1e-9, size=(nsteps, n))
    mine = [oracle.Solver(h, i) for i, h in enumerate(hs)]        # arrays the adapter's Hsolves borrow
    ref = [oracle.Solver(h, i) for i, h in enumerate(hs)]         # stepped by the reference's code
    rows = [np.array([int(h.compchips[h.ncompts - 1]) + 1], dtype=np.int32) for h in hs]
    vals = [np.zeros(1) for _ in hs]
    names = [b"/cell%d/solve" % i for i in range(n)]
    has_out = [i % 4 == 0 for i in range(n)]
    ptrs = []
    try:
        for i, (h, s) in enumerate(zip(hs, mine)):
            ncov = len(h.diff["covals0"]) if getattr(h, "diff", None) is not None and len(h.diff["nshells"]) else 0
            p = host.ah_create(C.addressof(s.s), names[i], len(s.stablist), ncov, 1, rows[i].ctypes.data,
                               vals[i].ctypes.data, int(has_out[i]))
            assert p
            ptrs.append(p)
        for p in ptrs:                    # RESET: every solver's init action
            assert host.ah_init(p) == 0
        dt = hs[0].dt
        for step in range(nsteps):
            for i in range(n):
                vals[i][0] = inj[step, i]
            for p in ptrs:                # the scheduler calls every hsolve in the step
                assert host.ah_process(p, step * dt) == 1
            for i, o in enumerate(ref):
                o.chip[rows[i][0]] = inj[step, i]
                o.run(1, "reference")
            for i in range(n):
                if has_out[i]:
                    np.testing.assert_array_equal(mine[i].vm, ref[i].vm)
            if step == 120:               # RESTORE2-style edit: sync, change Vm on the host, push
                host.ah_sync(ptrs[5])
                np.testing.assert_array_equal(mine[5].chip, ref[5].chip)
                mine[5].vm[:] += 1e-3
                ref[5].vm[:] += 1e-3
                assert host.ah_push(ptrs[5]) == 0
        for p in ptrs:
            host.ah_sync(p)
        for s, o in zip(mine, ref):
            np.testing.assert_array_equal(s.vm, o.vm)
            np.testing.assert_array_equal(s.chip, o.chip)
            np.testing.assert_array_equal(s.conc[:s.s.nconcs], o.conc[:o.s.nconcs])
    finally:
        arr = (C.c_void_p * len(ptrs))(*ptrs)
        host.ah_destroy_all(arr, len(ptrs))


def _save2(s):
    """The SAVE2 image of a solver (hines.c:553-558): n = nchips + ncompts +
    nconcs as an int, then chip[], vm[], conc[] as doubles."""
    nconc = s.s.nconcs
    n = len(s.chip) + len(s.vm) + nconc
    return (np.array([n], dtype=np.int32).tobytes() + s.chip.tobytes() + s.vm.tobytes() +
            s.conc[:nconc].tobytes())


def _restore2(s, image):
    """RESTORE2 (hines.c:560-571) into the solver's arrays."""
    nconc = s.s.nconcs
    n = int(np.frombuffer(image[:4], dtype=np.int32)[0])
    assert n == len(s.chip) + len(s.vm) + nconc
    d = np.frombuffer(image[4:], dtype=np.float64)
    s.chip[:] = d[:len(s.chip)]
    s.vm[:] = d[len(s.chip):len(s.chip) + len(s.vm)]
    s.conc[:nconc] = d[len(s.chip) + len(s.vm):]


@pytest.mark.gpu
def test_adapter_save2_restore2(tmp_path, oracle, gpu_engine):
    """SAVE2 after gbh_sync_chip writes the same bytes as the reference's own
    step code after the same steps; a RESTORE2 image (taken from the
    reference run 60 steps earlier) pushed into the running batch with
    gbh_push_state continues exactly as the reference continues from it."""
    host = _host_lib(tmp_path)
    n, dt = 12, None
    hs = [model.build(m) for m in configs.random_trees(n, size_range=(8, 48), seed=35)]
    mine = [oracle.Solver(h, i) for i, h in enumerate(hs)]
    ref = [oracle.Solver(h, i) for i, h in enumerate(hs)]
    zero = np.zeros(1, dtype=np.int32)
    nov = np.zeros(1)
    ptrs = []
    try:
        for i, s in enumerate(mine):
            h = hs[i]
            ncov = len(h.diff["covals0"]) if getattr(h, "diff", None) is not None and len(h.diff["nshells"]) else 0
            ptrs.append(host.ah_create(C.addressof(s.s), b"/c%d" % i, len(s.stablist), ncov, 0, zero.ctypes.data,
                                       nov.ctypes.data, 0))
        for p in ptrs:
            assert host.ah_init(p) == 0
        dt = hs[0].dt
        saved = None
        for step in range(200):
            for p in ptrs:
                assert host.ah_process(p, step * dt) == 1
            for o in ref:
                o.run(1, "reference")
            if step == 59:
                saved = [_save2(o) for o in ref]          # the reference's SAVE2 at step 60
            if step == 119:
                for p in ptrs:
                    host.ah_sync(p)                       # SAVE2 reads the host arrays
                for s, o in zip(mine, ref):
                    assert _save2(s) == _save2(o)
                for i, (s, o) in enumerate(zip(mine, ref)):
                    _restore2(s, saved[i])                # RESTORE2 of the step-60 image into both
                    _restore2(o, saved[i])
                    assert host.ah_push(ptrs[i]) == 0
        for p in ptrs:
            host.ah_sync(p)
        for s, o in zip(mine, ref):
            assert _save2(s) == _save2(o)
    finally:
        arr = (C.c_void_p * len(ptrs))(*ptrs)
        host.ah_destroy_all(arr, len(ptrs))
