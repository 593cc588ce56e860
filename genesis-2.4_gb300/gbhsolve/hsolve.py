"""ctypes mirror of the hsolve-level ABI (include/gbh_hsolve.h): GENESIS
hsolve elements registered one by one and stepped together by one batch
engine, as the GENESIS side does it for `chanmode` 4/5 solvers (the role of
the reference's per-hsolve registry, genesis/src/hines/cuda/cuda_hsolve.c:
64-145). Arrays are borrowed: keep the Solver objects alive while the
registry uses them.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, List, Optional, Sequence

import numpy as np

from . import engine as _eng

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
VALUE_FN = C.CFUNCTYPE(C.c_double, C.c_void_p)
SPIKE_FN = C.CFUNCTYPE(None, C.c_void_p)


class HsInput(C.Structure):
    _fields_ = [("kind", C.c_int), ("index", C.c_int64), ("sa", C.c_double), ("sb", C.c_double),
                ("value", VALUE_FN), ("ctx", C.c_void_p)]


class HsSynapse(C.Structure):
    _fields_ = [("target", C.c_int), ("target_op", C.c_int), ("weight", C.c_double), ("delay_steps", C.c_int)]


class HsSolver(C.Structure):
    _fields_ = [("dt", C.c_double), ("method", C.c_int), ("chanmode", C.c_int), ("calcmode", C.c_int),
                ("storemode", C.c_int), ("ncompts", C.c_int),
                ("nops", C.c_int), ("ops", _ip), ("nchips", C.c_int), ("chip", _dp),
                ("nfuncs", C.c_int), ("funcs", _ip), ("nravals", C.c_int), ("ravals", _dp),
                ("vm", _dp), ("ngivals", C.c_int), ("givals", _dp), ("nstab", C.c_int), ("stablist", _dp),
                ("nconcs", C.c_int), ("conc", _dp), ("nconcops", C.c_int), ("concops", _ip),
                ("nconcchips", C.c_int), ("concchip", _dp), ("tables", _eng.GbhTables),
                ("ndiffs", C.c_int), ("dconc", _ip), ("nshells", _ip), ("nshrows", _ip), ("nshfix", _ip),
                ("fbufval", _ip), ("ncovals0", C.c_int), ("covals0", _dp), ("nbufvals", C.c_int),
                ("bufvals", _dp), ("nelm_names", C.c_int), ("itotal", _dp),
                ("ninputs", C.c_int), ("inputs", C.POINTER(HsInput)), ("has_outputs", C.c_int),
                ("nsynapses", C.c_int), ("synapses", C.POINTER(HsSynapse)),
                ("on_spike", SPIKE_FN), ("spike_ctx", C.c_void_p)]


def _lib():
    lib = _eng.load()
    if not getattr(lib, "_hs_ready", False):
        lib.gbh_hs_register.argtypes = [C.POINTER(HsSolver)]
        lib.gbh_hs_step.argtypes = [C.c_int, C.c_longlong]
        lib.gbh_hs_sync.argtypes = [C.c_int]
        lib.gbh_hs_push.argtypes = [C.c_int]
        lib.gbh_hs_stats.argtypes = [C.POINTER(_eng.GbhStats)]
        lib.gbh_hs_cleanup.restype = None
        lib._hs_ready = True
    return lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None and a.size else C.cast(0, t)


class Solver:
    """One hsolve's arrays (owned here, as GENESIS owns an Hsolve's) and its
    registration. inputs: list of (kind, index, sa, sb, value_fn) with
    value_fn() -> float read at every step; synapses: list of (target id,
    target op, weight, delay steps); on_spike: called for every spike."""

    def __init__(self, h, inputs: Sequence = (), synapses: Sequence = (), has_outputs: bool = False,
                 on_spike: Optional[Callable[[], None]] = None):
        self.h = h
        self.ops = np.array(h.ops, dtype=np.int32)
        self.chip = np.array(h.chip, dtype=np.float64)
        self.funcs = np.array(h.funcs, dtype=np.int32)
        self.ravals = np.array(h.ravals, dtype=np.float64)
        self.vm = np.array(h.vm, dtype=np.float64)
        self.givals = np.array(h.givals, dtype=np.float64)
        self.stablist = np.array(h.stablist, dtype=np.float64)
        self.conc = np.array(h.conc, dtype=np.float64)
        self.concops = np.array(h.concops, dtype=np.int32)
        self.concchip = np.array(h.concchip, dtype=np.float64)
        self.tablist = np.ascontiguousarray(h.tablist, dtype=np.float64)
        self.xvals = np.ascontiguousarray(h.xvals, dtype=np.float64)
        self.yvals = np.ascontiguousarray(h.yvals, dtype=np.float64)
        s = HsSolver()
        s.dt, s.method, s.chanmode, s.calcmode = h.dt, h.method, h.chanmode, h.calcmode
        s.storemode = 0
        s.ncompts = h.ncompts
        s.nops, s.ops = len(self.ops), _p(self.ops, _ip)
        s.nchips, s.chip = len(self.chip), _p(self.chip, _dp)
        s.nfuncs, s.funcs = len(self.funcs), _p(self.funcs, _ip)
        s.nravals, s.ravals = len(self.ravals), _p(self.ravals, _dp)
        s.vm = _p(self.vm, _dp)
        s.ngivals, s.givals = len(self.givals), _p(self.givals, _dp)
        s.nstab, s.stablist = len(self.stablist), _p(self.stablist, _dp)
        s.nconcs, s.conc = len(self.conc), _p(self.conc, _dp)
        s.nconcops, s.concops = len(self.concops), _p(self.concops, _ip)
        s.nconcchips, s.concchip = len(self.concchip), _p(self.concchip, _dp)
        t = s.tables
        t.ncols, t.xdivs, t.ydivs = h.ncols, h.xdivs, h.ydivs
        t.xmin, t.invdx, t.ymin, t.invdy = h.xmin, h.invdx, h.ymin, h.invdy
        t.tablist, t.xvals, t.yvals = _p(self.tablist, _dp), _p(self.xvals, _dp), _p(self.yvals, _dp)
        self._value_fns = []
        self._inputs = (HsInput * max(1, len(inputs)))()
        for k, (kind, index, sa, sb, fn) in enumerate(inputs):
            cb = VALUE_FN(lambda ctx, fn=fn: float(fn()))
            self._value_fns.append(cb)
            self._inputs[k] = HsInput(kind, index, sa, sb, cb, None)
        s.ninputs, s.inputs = len(inputs), self._inputs
        s.has_outputs = 1 if has_outputs else 0
        self._syn = (HsSynapse * max(1, len(synapses)))()
        for k, (tgt, op, w, d) in enumerate(synapses):
            self._syn[k] = HsSynapse(int(tgt), int(op), float(w), int(d))
        s.nsynapses, s.synapses = len(synapses), self._syn
        self._spike_cb = SPIKE_FN(lambda ctx: on_spike()) if on_spike else SPIKE_FN()
        s.on_spike = self._spike_cb
        self.s = s
        self.id = -1

    def register(self) -> int:
        self.id = _lib().gbh_hs_register(C.byref(self.s))
        if self.id < 0:
            raise RuntimeError("gbh_hs_register failed")
        return self.id

    def step(self, stamp: int) -> int:
        rc = _lib().gbh_hs_step(self.id, int(stamp))
        if rc < 0:
            raise RuntimeError("gbh_hs_step: %s" % _lib().gbh_last_error().decode())
        return rc

    def sync(self) -> None:
        if _lib().gbh_hs_sync(self.id) != 0:
            raise RuntimeError("gbh_hs_sync failed")

    def push(self) -> None:
        if _lib().gbh_hs_push(self.id) != 0:
            raise RuntimeError("gbh_hs_push failed")


def stats() -> _eng.GbhStats:
    st = _eng.GbhStats()
    if _lib().gbh_hs_stats(C.byref(st)) != 0:
        raise RuntimeError("no batch engine")
    return st


def cleanup() -> None:
    _lib().gbh_hs_cleanup()
