"""ctypes binding of the CPU oracle (liboracle.so) and, where it was built, of
the reference's own step code (oracle/_ref/libhsolve_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, never by the engine package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_ORACLE = os.path.join(HERE, "liboracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libhsolve_ref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
SPIKE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int)
SYN_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int)


class OrcSolver(C.Structure):
    """Mirror of struct orc_solver (hsolve_oracle.h)."""
    _fields_ = [
        ("id", C.c_int),
        ("ncompts", C.c_int), ("nchips", C.c_int), ("nops", C.c_int),
        ("nfuncs", C.c_int), ("nravals", C.c_int), ("ngivals", C.c_int),
        ("ops", _ip), ("chip", _dp), ("funcs", _ip), ("ravals", _dp),
        ("results", _dp), ("vm", _dp), ("givals", _dp),
        ("chanmode", C.c_int), ("calcmode", C.c_int), ("storemode", C.c_int),
        ("crank", C.c_int), ("dt", C.c_double),
        ("ncols", C.c_int), ("xdivs", C.c_int), ("ydivs", C.c_int),
        ("xmin", C.c_double), ("invdx", C.c_double), ("ymin", C.c_double), ("invdy", C.c_double),
        ("tablist", _dp), ("xvals", _dp), ("yvals", _dp), ("stablist", _dp),
        ("nconcs", C.c_int),
        ("conc", _dp), ("flux", _dp), ("codiag", _dp), ("coresult", _dp),
        ("nconcchips", C.c_int), ("nconcops", C.c_int),
        ("concops", _ip), ("concchip", _dp), ("ovals", _dp),
        ("ndiffs", C.c_int), ("dconc", _ip), ("nshells", _ip), ("nshrows", _ip), ("nshfix", _ip),
        ("fbufval", _ip), ("covals0", _dp), ("bufvals", _dp), ("covals", _dp), ("cores", _dp),
        ("nconcchips_used", C.c_int),
        ("itotal", _dp), ("nelm_names", C.c_int),
        ("childops", _ip), ("childchips", _ip),
        ("on_spike", SPIKE_FN), ("on_syn", SYN_FN), ("hook_ctx", C.c_void_p),
        ("err_op", C.c_int),
    ]


def ensure_built(with_reference: bool = True) -> None:
    """Builds liboracle.so (and the reference binding when its sources exist)."""
    need = not os.path.exists(LIB_ORACLE)
    src = [os.path.join(HERE, f) for f in ("hsolve_oracle.c", "hsolve_oracle.h", "ref_shim.c")]
    if not need:
        t = os.path.getmtime(LIB_ORACLE)
        need = any(os.path.getmtime(s) > t for s in src)
    if need or (with_reference and reference_sources_present() and not os.path.exists(LIB_REF)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)


_ref_src = None


def reference_src() -> str:
    """The reference's genesis/src directory: GENESIS_REF_SRC in the
    environment, else the default that oracle/Makefile builds from."""
    global _ref_src
    if _ref_src is None:
        env = os.environ.get("GENESIS_REF_SRC")
        if env:
            _ref_src = env
        else:
            r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
            _ref_src = r.stdout.strip() if r.returncode == 0 else ""
    return _ref_src


def reference_sources_present() -> bool:
    src = reference_src()
    return bool(src) and os.path.exists(os.path.join(src, "hines", "hines_chip.c"))


_libs = {}


def seed_rng(seed: int, impl: str = "oracle") -> None:
    """Seeds SYN3_OP's generator (G_SEEDRNG) of the oracle or of the
    reference's own code."""
    lib = _lib(impl)
    (lib.orc_seed_rng if impl == "oracle" else lib.G_SEEDRNG)(int(seed))


def _lib(which: str):
    if which not in _libs:
        path = LIB_ORACLE if which == "oracle" else LIB_REF
        lib = C.CDLL(path)
        if which == "oracle":
            lib.orc_process.argtypes = [C.POINTER(OrcSolver)]
            lib.orc_run.argtypes = [C.POINTER(OrcSolver), C.c_int]
            lib.orc_run_loss.argtypes = [C.POINTER(OrcSolver), C.c_int, C.c_int, _ip, _dp, _dp]
            lib.orc_run_trace.argtypes = [C.POINTER(OrcSolver), C.c_int, C.c_int, _ip, _dp, _ip]
            lib.orc_net_create.restype = C.c_void_p
            lib.orc_net_create.argtypes = [C.c_int, C.POINTER(C.POINTER(OrcSolver)), _ip, _ip, _ip,
                                           _ip, _dp, _ip]
            lib.orc_net_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_longlong)]
            lib.orc_net_destroy.argtypes = [C.c_void_p]
            lib.orc_net_set_process.argtypes = [C.c_void_p, C.c_void_p]
            lib.orc_net_deliver.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip, _dp, C.POINTER(C.c_longlong)]
            lib.orc_net_step_count.restype = C.c_longlong
            lib.orc_net_step_count.argtypes = [C.c_void_p]
            lib.orc_seed_rng.argtypes = [C.c_long]
            lib.orc_seed_rng.restype = None
        else:
            lib.ref_process.argtypes = [C.POINTER(OrcSolver)]
            lib.ref_run.argtypes = [C.POINTER(OrcSolver), C.c_int]
            lib.G_SEEDRNG.argtypes = [C.c_long]
            lib.G_SEEDRNG.restype = None
        _libs[which] = lib
    return _libs[which]


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None and a.size else C.cast(0, t)


class Solver:
    """One hsolve's arrays owned by numpy, wrapped in an OrcSolver."""

    def __init__(self, arrays, sid: int = 0):
        h = arrays
        self.h = h
        self.ops = np.array(h.ops, dtype=np.int32, copy=True)
        self.chip = np.array(h.chip, dtype=np.float64, copy=True)
        self.funcs = np.array(h.funcs, dtype=np.int32, copy=True)
        self.ravals = np.array(h.ravals, dtype=np.float64, copy=True)
        self.results = np.zeros(2 * h.ncompts, dtype=np.float64)
        self.vm = np.array(h.vm, dtype=np.float64, copy=True)
        self.givals = np.array(h.givals, dtype=np.float64, copy=True)
        self.tablist = np.array(h.tablist, dtype=np.float64, copy=True)
        self.xvals = np.array(h.xvals, dtype=np.float64, copy=True)
        self.yvals = np.array(h.yvals, dtype=np.float64, copy=True)
        self.stablist = np.array(h.stablist, dtype=np.float64, copy=True)
        nconc = max(len(h.conc), 1)
        self.conc = np.zeros(nconc + 1, dtype=np.float64)
        self.conc[:len(h.conc)] = h.conc
        self.flux = np.zeros(nconc + 1, dtype=np.float64)
        self.codiag = np.ones(nconc + 1, dtype=np.float64)
        self.coresult = np.zeros(nconc + 1, dtype=np.float64)
        self.concops = np.array(h.concops, dtype=np.int32, copy=True)
        self.concchip = np.array(h.concchip, dtype=np.float64, copy=True)
        self.childops = np.array(h.childops, dtype=np.int32, copy=True)
        self.childchips = np.array(h.childchips, dtype=np.int32, copy=True)
        s = OrcSolver()
        s.id = sid
        s.ncompts = h.ncompts
        s.nchips = len(self.chip)
        s.nops = len(self.ops)
        s.nfuncs = len(self.funcs)
        s.nravals = len(self.ravals)
        s.ngivals = len(self.givals)
        s.ops, s.chip, s.funcs = _p(self.ops, _ip), _p(self.chip, _dp), _p(self.funcs, _ip)
        s.ravals, s.results, s.vm = _p(self.ravals, _dp), _p(self.results, _dp), _p(self.vm, _dp)
        s.givals = _p(self.givals, _dp)
        s.chanmode, s.calcmode = h.chanmode, h.calcmode
        s.storemode = int(getattr(h, "storemode", 0))
        s.crank, s.dt = h.crank, h.dt
        s.ncols, s.xdivs, s.ydivs = h.ncols, h.xdivs, h.ydivs
        s.xmin, s.invdx, s.ymin, s.invdy = h.xmin, h.invdx, h.ymin, h.invdy
        s.tablist = _p(self.tablist, _dp) if h.ncols else C.cast(0, _dp)
        s.xvals, s.yvals = _p(self.xvals, _dp), _p(self.yvals, _dp)
        s.stablist = _p(self.stablist, _dp)
        s.nconcs = len(h.conc)
        s.conc, s.flux = _p(self.conc, _dp), _p(self.flux, _dp)
        s.codiag, s.coresult = _p(self.codiag, _dp), _p(self.coresult, _dp)
        s.nconcchips = len(self.concchip)
        s.nconcops = len(self.concops)
        s.concops, s.concchip = _p(self.concops, _ip), _p(self.concchip, _dp)
        # TAUPUMP_OP writes its 1/tau into ovals[] (hines_conc_chip.c:118-121)
        self.ovals = np.zeros(max(1, int(np.count_nonzero(self.concops == 11000))), dtype=np.float64)
        s.ovals = _p(self.ovals, _dp)
        diff = getattr(h, "diff", None)
        if diff is not None and len(diff["nshells"]):
            self.dconc, self.nshells, self.nshrows, self.nshfix, self.fbufval = (
                np.array(diff[k], dtype=np.int32, copy=True) for k in ("dconc", "nshells", "nshrows", "nshfix",
                                                                         "fbufval"))
            self.covals0 = np.array(diff["covals0"], dtype=np.float64, copy=True)
            self.bufvals = np.array(diff["bufvals"], dtype=np.float64, copy=True)
            w = self.nshells * self.nshrows
            self.covals = np.zeros(int(np.max(w * self.nshrows + self.nshrows)) + 1)
            self.cores = np.zeros(int(np.max(w)) + 1)
            s.ndiffs = len(self.nshells)
            s.dconc, s.nshells, s.nshrows = _p(self.dconc, _ip), _p(self.nshells, _ip), _p(self.nshrows, _ip)
            s.nshfix, s.fbufval = _p(self.nshfix, _ip), _p(self.fbufval, _ip)
            s.covals0, s.bufvals = _p(self.covals0, _dp), _p(self.bufvals, _dp)
            s.covals, s.cores = _p(self.covals, _dp), _p(self.cores, _dp)
        else:
            s.ndiffs = 0
        s.nconcchips_used = 1 if len(self.concchip) else 0
        # storemode: itotal[nelm_names] summed every step (hines_chip.c:134-166)
        self.itotal = np.zeros(max(int(getattr(h, "nelm_names", 0)), 1))
        s.itotal = _p(self.itotal, _dp) if s.storemode else C.cast(0, _dp)
        s.nelm_names = int(getattr(h, "nelm_names", 0)) if s.storemode else 0
        s.childops, s.childchips = _p(self.childops, _ip), _p(self.childchips, _ip)
        self.s = s

    def run(self, nsteps: int, impl: str = "oracle") -> None:
        lib = _lib(impl)
        fn = lib.orc_run if impl == "oracle" else lib.ref_run
        rc = fn(C.byref(self.s), int(nsteps))
        if rc != 0:
            raise RuntimeError("%s step failed at op %d" % (impl, self.s.err_op))


    def run_trace(self, nsteps: int, rows, table_rows: bool = False):
        """Runs nsteps steps; returns vm[rows] after every step (nsteps x
        len(rows)) and, with table_rows, every compartment's voltage-table
        row after every step (nsteps x ncompts), else None."""
        r = np.ascontiguousarray(rows, dtype=np.int32)
        out = np.empty((int(nsteps), len(r)))
        tr = np.empty((int(nsteps), self.h.ncompts), dtype=np.int32) if table_rows else None
        rc = _lib("oracle").orc_run_trace(C.byref(self.s), int(nsteps), len(r), _p(r, _ip), _p(out, _dp),
                                          _p(tr, _ip) if tr is not None else C.cast(0, _ip))
        if rc != 0:
            raise RuntimeError("oracle step failed at op %d" % self.s.err_op)
        return out, tr

    def run_loss(self, nsteps: int, rows, trace) -> float:
        """Runs nsteps steps; returns sum over steps and targets of
        (vm[row] after the step - trace[step][target])^2 (orc_run_loss)."""
        r = np.ascontiguousarray(rows, dtype=np.int32)
        tr = np.ascontiguousarray(trace, dtype=np.float64).reshape(int(nsteps), len(r))
        out = C.c_double(0.0)
        rc = _lib("oracle").orc_run_loss(C.byref(self.s), int(nsteps), len(r), _p(r, _ip), _p(tr, _dp),
                                         C.byref(out))
        if rc != 0:
            raise RuntimeError("oracle step failed at op %d" % self.s.err_op)
        return out.value


class Network:
    """Many single-hsolve solvers exchanging spike events (orc_net_*)."""

    def __init__(self, solvers, syn_start, tgt_solver, tgt_child, tgt_op, weight, delay_steps,
                 impl: str = "oracle"):
        self.solvers = solvers
        self.arr = (C.POINTER(OrcSolver) * len(solvers))(*[C.pointer(s.s) for s in solvers])
        self.syn_start = np.ascontiguousarray(syn_start, dtype=np.int32)
        self.tgt_solver = np.ascontiguousarray(tgt_solver, dtype=np.int32)
        self.tgt_child = np.ascontiguousarray(tgt_child, dtype=np.int32)
        self.tgt_op = np.ascontiguousarray(tgt_op, dtype=np.int32)
        self.weight = np.ascontiguousarray(weight, dtype=np.float64)
        self.delay = np.ascontiguousarray(delay_steps, dtype=np.int32)
        lib = _lib("oracle")
        self.lib = lib
        self.net = lib.orc_net_create(len(solvers), self.arr, _p(self.syn_start, _ip),
                                      _p(self.tgt_solver, _ip), _p(self.tgt_child, _ip),
                                      _p(self.tgt_op, _ip), _p(self.weight, _dp), _p(self.delay, _ip))
        if impl == "reference":
            ref = _lib("reference")
            lib.orc_net_set_process(self.net, C.cast(ref.ref_process, C.c_void_p))
        self.spikes = np.zeros(len(solvers), dtype=np.int64)

    def run(self, nsteps: int) -> None:
        rc = self.lib.orc_net_run(self.net, int(nsteps),
                                  self.spikes.ctypes.data_as(C.POINTER(C.c_longlong)))
        if rc != 0:
            raise RuntimeError("network step failed")

    @property
    def step(self) -> int:
        return int(self.lib.orc_net_step_count(self.net))

    def deliver(self, tgt_solver, tgt_child, tgt_op, weight, fire_step) -> None:
        """Events from outside the network (orc_net_deliver)."""
        a = [np.ascontiguousarray(x, dtype=np.int32) for x in (tgt_solver, tgt_child, tgt_op)]
        w = np.ascontiguousarray(weight, dtype=np.float64)
        f = np.ascontiguousarray(fire_step, dtype=np.int64)
        if len(w):
            self.lib.orc_net_deliver(self.net, len(w), _p(a[0], _ip), _p(a[1], _ip), _p(a[2], _ip), _p(w, _dp),
                                     f.ctypes.data_as(C.POINTER(C.c_longlong)))

    def __del__(self):
        try:
            self.lib.orc_net_destroy(self.net)
        except Exception:
            pass
