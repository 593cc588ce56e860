"""ctypes binding of the C ABI in include/gbhsolve.h (libgbhsolve.so).

This is the host-side mirror of the reference's accelerator interface for
the hsolve chanmode 4/5 step (genesis/src/hines/cuda/cuda_hsolve.h:22-25):
``Engine(solvers)`` plays ``cuda_init``, ``Engine.run`` plays the multiloop
``cuda_chip_update`` returning "vm ready", ``get_state`` plays
``cuda_sync_chip``, and ``close`` plays ``cuda_cleanup``. There is no CPU
fallback: if the library cannot be loaded or the model uses something the
engine does not implement, an exception is raised.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional, Sequence

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_int64)

ABI_VERSION = 4
PREC_FP64, PREC_MIXED = 0, 1
IN_SET, IN_ADD, IN_FLUX = 0, 1, 2     # gbh_register_inputs_typed kinds


class GbhError(C.Structure):
    _fields_ = [("code", C.c_int), ("solver", C.c_int), ("row", C.c_int), ("opcode", C.c_int),
                ("position", C.c_int), ("message", C.c_char * 256)]


class GbhTables(C.Structure):
    _fields_ = [("ncols", C.c_int), ("xdivs", C.c_int), ("ydivs", C.c_int),
                ("xmin", C.c_double), ("invdx", C.c_double), ("ymin", C.c_double),
                ("invdy", C.c_double), ("tablist", _dp), ("xvals", _dp), ("yvals", _dp)]


class GbhBatchDesc(C.Structure):
    _fields_ = [("abi_version", C.c_int), ("nsolvers", C.c_int), ("dt", C.c_double),
                ("method", _ip), ("chanmode", _ip), ("calcmode", _ip), ("table_set", _ip),
                ("ntables", C.c_int), ("tables", C.POINTER(GbhTables)),
                ("ops_start", _lp), ("ops", _ip),
                ("chip_start", _lp), ("chip", _dp),
                ("funcs_start", _lp), ("funcs", _ip),
                ("ravals_start", _lp), ("ravals", _dp),
                ("vm_start", _lp), ("vm", _dp),
                ("givals_start", _lp), ("givals", _dp),
                ("stab_start", _lp), ("stablist", _dp),
                ("conc_start", _lp), ("conc", _dp),
                ("concops_start", _lp), ("concops", _ip),
                ("concchip_start", _lp), ("concchip", _dp),
                ("diff_start", _lp), ("dconc", _ip), ("nshells", _ip), ("nshrows", _ip), ("nshfix", _ip),
                ("fbufval", _ip), ("covals0_start", _lp), ("covals0", _dp), ("bufvals_start", _lp),
                ("bufvals", _dp), ("storemode", _ip), ("itotal_start", _lp)]


class GbhSynapses(C.Structure):
    _fields_ = [("nsynapses", C.c_int64), ("src_start", _lp), ("target_solver", _ip),
                ("target_op", _ip), ("weight", _dp), ("delay_steps", _ip)]


class GbhRemoteSynapses(C.Structure):
    _fields_ = [("nsources", C.c_int), ("src_start", _lp), ("target_solver", _ip), ("target_op", _ip),
                ("weight", _dp), ("delay_steps", _ip), ("first_solver", C.c_int64)]


class GbhOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("steps_per_launch", C.c_int),
                ("warps_per_block", C.c_int), ("use_graph", C.c_int), ("device", C.c_int),
                ("jit", C.c_int), ("wide_min", C.c_int)]


class GbhLossSpec(C.Structure):
    _fields_ = [("ntargets", C.c_int), ("solver", _ip), ("row", _ip), ("trace", _dp)]


class GbhStats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("device_ms", C.c_double), ("compartments", C.c_int64),
                ("tiles", C.c_int64), ("launches", C.c_int64), ("bytes_per_step", C.c_double),
                ("steps_per_launch", C.c_int), ("warps_per_block", C.c_int), ("precision", C.c_int),
                ("jit_kernels", C.c_int), ("jit_min_blocks", C.c_int),
                ("grad_forward_ms", C.c_double), ("grad_reverse_ms", C.c_double), ("jit_compact", C.c_int),
                ("cooperative", C.c_int), ("wide_tiles", C.c_int64), ("stack_tiles", C.c_int64),
                ("grad_kept_steps", C.c_int64)]


EXPORTED = ["gbh_jit_source", "gbh_validate", "gbh_create", "gbh_run", "gbh_run_async", "gbh_get_state", "gbh_set_state",
            "gbh_enable_givals", "gbh_get_givals", "gbh_register_inputs", "gbh_set_inputs_async",
            "gbh_register_outputs", "gbh_get_outputs_async", "gbh_get_spike_counts", "gbh_get_stats",
            "gbh_destroy", "gbh_last_error", "gbh_run_noalloc", "gbh_loss_gradient", "gbh_create_dist",
            "gbh_get_spiked", "gbh_deliver_remote", "gbh_step_io", "gbh_io_sync", "gbh_run_io",
            "gbh_register_inputs_typed", "gbh_get_itotal",
            # hsolve-level ABI (include/gbh_hsolve.h, mirrored in gbhsolve/hsolve.py)
            "gbh_hs_register", "gbh_hs_set_synapses", "gbh_hs_step", "gbh_hs_sync", "gbh_hs_push",
            "gbh_hs_stats", "gbh_hs_count", "gbh_hs_cleanup"]

_LIB = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads libgbhsolve.so (building it first when sources are newer)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if build_if_missing:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError("libgbhsolve.so is missing; run gbhsolve.build.build()")
    lib = C.CDLL(_build.LIB)
    lib.gbh_create.restype = C.c_void_p
    lib.gbh_create.argtypes = [C.POINTER(GbhBatchDesc), C.POINTER(GbhSynapses), C.POINTER(GbhOptions),
                               C.POINTER(GbhError)]
    lib.gbh_jit_source.restype = C.c_int64
    lib.gbh_jit_source.argtypes = [C.POINTER(GbhBatchDesc), C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_int64]
    lib.gbh_validate.argtypes = [C.POINTER(GbhBatchDesc), C.POINTER(GbhError), _lp, _lp]
    lib.gbh_run.argtypes = [C.c_void_p, C.c_int]
    lib.gbh_run_async.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    lib.gbh_get_state.argtypes = [C.c_void_p, _dp, _dp, _dp, _ip]
    lib.gbh_set_state.argtypes = [C.c_void_p, _dp, _dp, _dp]
    lib.gbh_enable_givals.argtypes = [C.c_void_p, C.c_int]
    lib.gbh_get_givals.argtypes = [C.c_void_p, _dp]
    lib.gbh_get_spike_counts.argtypes = [C.c_void_p, _lp]
    lib.gbh_register_inputs.argtypes = [C.c_void_p, C.c_int, _ip, _lp]
    lib.gbh_set_inputs_async.argtypes = [C.c_void_p, _dp, C.c_void_p]
    lib.gbh_register_outputs.argtypes = [C.c_void_p, C.c_int, _ip, _ip]
    lib.gbh_get_outputs_async.argtypes = [C.c_void_p, _dp, C.c_void_p]
    lib.gbh_get_stats.argtypes = [C.c_void_p, C.POINTER(GbhStats)]
    lib.gbh_destroy.argtypes = [C.c_void_p]
    lib.gbh_last_error.restype = C.c_char_p
    lib.gbh_run_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    lib.gbh_create_dist.restype = C.c_void_p
    lib.gbh_create_dist.argtypes = [C.POINTER(GbhBatchDesc), C.POINTER(GbhSynapses), C.POINTER(GbhRemoteSynapses),
                                    C.POINTER(GbhOptions), C.POINTER(GbhError)]
    lib.gbh_get_spiked.argtypes = [C.c_void_p, C.POINTER(C.c_uint8)]
    lib.gbh_deliver_remote.argtypes = [C.c_void_p, C.POINTER(C.c_uint8)]
    lib.gbh_step_io.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_void_p]
    lib.gbh_io_sync.argtypes = [C.c_void_p]
    lib.gbh_run_io.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_int, C.c_void_p]
    lib.gbh_register_inputs_typed.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _lp, _dp, _dp]
    lib.gbh_loss_gradient.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(GbhLossSpec), _dp, _dp, _dp, _dp]
    _LIB = lib
    return lib


def _cat(arrays, dtype):
    starts = np.zeros(len(arrays) + 1, dtype=np.int64)
    for i, a in enumerate(arrays):
        starts[i + 1] = starts[i] + len(a)
    flat = np.concatenate([np.asarray(a, dtype=dtype) for a in arrays]) if starts[-1] else \
        np.zeros(1, dtype=dtype)
    return starts, np.ascontiguousarray(flat)


def _ptr(a, t):
    return a.ctypes.data_as(t)


class EngineError(RuntimeError):
    def __init__(self, err: GbhError):
        self.code = err.code
        self.solver = err.solver
        self.row = err.row
        self.opcode = err.opcode
        self.position = err.position
        super().__init__("gbh_create failed (code %d, solver %d, row %d, opcode %d, pos %d): %s" % (
            err.code, err.solver, err.row, err.opcode, err.position, err.message.decode()))


class Batch:
    """Concatenated reference arrays of many hsolve elements (plain numpy)."""

    def __init__(self, solvers: Sequence, synapses: Optional[dict] = None):
        self.solvers = list(solvers)
        s0 = self.solvers[0]
        dt = s0.dt
        for s in self.solvers:
            if s.dt != dt:
                raise ValueError("all solvers of a batch share dt")
        self.dt = dt
        self.n = len(self.solvers)
        # table sets: share identical tables
        self.table_keys = {}
        self.table_list = []
        ts = []
        content = {}
        for s in self.solvers:
            key = id(s.tablist)
            if key not in content:
                tab = np.ascontiguousarray(s.tablist)
                content[key] = (s.ncols, s.xdivs, s.ydivs, s.xmin, s.invdx, s.ymin, s.invdy,
                                hash(tab.tobytes()), hash(np.ascontiguousarray(s.xvals).tobytes()),
                                hash(np.ascontiguousarray(s.yvals).tobytes()))
            key = content[key]      # identical tables share one table set
            if key not in self.table_keys:
                self.table_keys[key] = len(self.table_list)
                self.table_list.append(s)
            ts.append(self.table_keys[key])
        self.table_set = np.array(ts, dtype=np.int32)
        self.method = np.array([s.method for s in self.solvers], dtype=np.int32)
        self.chanmode = np.array([s.chanmode for s in self.solvers], dtype=np.int32)
        self.calcmode = np.array([s.calcmode for s in self.solvers], dtype=np.int32)
        self.ops_start, self.ops = _cat([s.ops for s in self.solvers], np.int32)
        self.chip_start, self.chip = _cat([s.chip for s in self.solvers], np.float64)
        self.funcs_start, self.funcs = _cat([s.funcs for s in self.solvers], np.int32)
        self.ravals_start, self.ravals = _cat([s.ravals for s in self.solvers], np.float64)
        self.vm_start, self.vm = _cat([s.vm for s in self.solvers], np.float64)
        self.givals_start, self.givals = _cat([s.givals for s in self.solvers], np.float64)
        self.stab_start, self.stablist = _cat([s.stablist for s in self.solvers], np.float64)
        self.conc_start, self.conc = _cat([s.conc for s in self.solvers], np.float64)
        self.concops_start, self.concops = _cat([s.concops for s in self.solvers], np.int32)
        self.concchip_start, self.concchip = _cat([s.concchip for s in self.solvers], np.float64)
        self._tables = (GbhTables * max(1, len(self.table_list)))()
        self._keep = []
        for k, s in enumerate(self.table_list):
            t = self._tables[k]
            t.ncols, t.xdivs, t.ydivs = s.ncols, s.xdivs, s.ydivs
            t.xmin, t.invdx, t.ymin, t.invdy = s.xmin, s.invdx, s.ymin, s.invdy
            tab = np.ascontiguousarray(s.tablist, dtype=np.float64)
            xv = np.ascontiguousarray(s.xvals, dtype=np.float64)
            yv = np.ascontiguousarray(s.yvals, dtype=np.float64)
            self._keep += [tab, xv, yv]
            t.tablist = _ptr(tab, _dp) if tab.size else C.cast(0, _dp)
            t.xvals = _ptr(xv, _dp) if xv.size else C.cast(0, _dp)
            t.yvals = _ptr(yv, _dp) if yv.size else C.cast(0, _dp)
        d = GbhBatchDesc()
        d.abi_version = ABI_VERSION
        d.nsolvers = self.n
        d.dt = dt
        d.method, d.chanmode = _ptr(self.method, _ip), _ptr(self.chanmode, _ip)
        d.calcmode, d.table_set = _ptr(self.calcmode, _ip), _ptr(self.table_set, _ip)
        d.ntables = len(self.table_list)
        d.tables = self._tables
        for name, t in (("ops", _ip), ("chip", _dp), ("funcs", _ip), ("ravals", _dp), ("vm", _dp),
                        ("givals", _dp), ("stablist", _dp), ("conc", _dp), ("concops", _ip),
                        ("concchip", _dp)):
            start = "stab_start" if name == "stablist" else name + "_start"
            setattr(d, start, _ptr(getattr(self, start), _lp))
            setattr(d, name, _ptr(getattr(self, name), t))
        # diffusion systems (optional `diff` dict on a solver)
        diffs = [getattr(s, "diff", None) for s in self.solvers]
        if any(x is not None and len(x["nshells"]) for x in diffs):
            empty = dict(dconc=[], nshells=[], nshrows=[], nshfix=[], fbufval=[], covals0=[], bufvals=[])
            diffs = [x if x is not None else empty for x in diffs]
            self.diff_start, self.dconc = _cat([x["dconc"] for x in diffs], np.int32)
            for k in ("nshells", "nshrows", "nshfix", "fbufval"):
                setattr(self, k, _cat([x[k] for x in diffs], np.int32)[1])
            self.covals0_start, self.covals0 = _cat([x["covals0"] for x in diffs], np.float64)
            self.bufvals_start, self.bufvals = _cat([x["bufvals"] for x in diffs], np.float64)
            d.diff_start = _ptr(self.diff_start, _lp)
            for k in ("dconc", "nshells", "nshrows", "nshfix", "fbufval"):
                setattr(d, k, _ptr(getattr(self, k), _ip))
            d.covals0_start, d.covals0 = _ptr(self.covals0_start, _lp), _ptr(self.covals0, _dp)
            d.bufvals_start, d.bufvals = _ptr(self.bufvals_start, _lp), _ptr(self.bufvals, _dp)
        # storemode (optional `storemode` / `nelm_names` on a solver)
        self.storemode = np.array([int(getattr(s, "storemode", 0)) for s in self.solvers], dtype=np.int32)
        nelm = [int(getattr(s, "nelm_names", 0)) if m else 0 for s, m in zip(self.solvers, self.storemode)]
        self.itotal_start = np.concatenate([[0], np.cumsum(nelm)]).astype(np.int64)
        if self.storemode.any():
            d.storemode, d.itotal_start = _ptr(self.storemode, _ip), _ptr(self.itotal_start, _lp)
        self.desc = d
        self.syn = None
        if synapses is not None:
            self._syn = {k: np.ascontiguousarray(v) for k, v in synapses.items()}
            sy = GbhSynapses()
            sy.nsynapses = len(self._syn["target_solver"])
            sy.src_start = _ptr(self._syn["src_start"].astype(np.int64), _lp)
            self._syn["src_start"] = self._syn["src_start"].astype(np.int64)
            sy.src_start = _ptr(self._syn["src_start"], _lp)
            self._syn["target_solver"] = self._syn["target_solver"].astype(np.int32)
            self._syn["target_op"] = self._syn["target_op"].astype(np.int32)
            self._syn["weight"] = self._syn["weight"].astype(np.float64)
            self._syn["delay_steps"] = self._syn["delay_steps"].astype(np.int32)
            sy.target_solver = _ptr(self._syn["target_solver"], _ip)
            sy.target_op = _ptr(self._syn["target_op"], _ip)
            sy.weight = _ptr(self._syn["weight"], _dp)
            sy.delay_steps = _ptr(self._syn["delay_steps"], _ip)
            self.syn = sy

    def split(self, flat, starts):
        return [flat[starts[i]:starts[i + 1]] for i in range(self.n)]


def validate(solvers: Sequence):
    """Host-only decode of a batch; returns (neurons, tile types) or raises."""
    lib = load()
    b = Batch(solvers)
    err = GbhError()
    nn = C.c_int64(0)
    nt = C.c_int64(0)
    rc = lib.gbh_validate(C.byref(b.desc), C.byref(err), C.byref(nn), C.byref(nt))
    if rc != 0:
        raise EngineError(err)
    return nn.value, nt.value


def jit_source(solvers: Sequence, precision: int = PREC_FP64, type_index: int = 0, compact: int = 0) -> str:
    """CUDA source generated for one tile type (host only, no GPU).

    compact: 0 (or False) unrolled form, 1 (or True) compact looped form,
    2 unrolled form with the eliminated rows in shared memory."""
    lib = load()
    b = Batch(solvers)
    n = lib.gbh_jit_source(C.byref(b.desc), precision, type_index, int(compact), None, 0)
    if n < 0:
        raise RuntimeError("gbh_jit_source failed: %s" % lib.gbh_last_error().decode())
    buf = C.create_string_buffer(int(n) + 1)
    lib.gbh_jit_source(C.byref(b.desc), precision, type_index, int(compact), buf, int(n) + 1)
    return buf.value.decode()


class Engine:
    """A device engine over a batch of hsolve elements."""

    def __init__(self, solvers: Sequence, synapses: Optional[dict] = None, precision: int = PREC_FP64,
                 steps_per_launch: int = 0, warps_per_block: int = 0, device: int = 0, jit: bool = True,
                 use_graph: bool = False, remote: Optional[dict] = None, wide_min: int = 0):
        self.lib = load()
        self.batch = Batch(solvers, synapses)
        # jit: True (autotuned forms), False (interpreter), or the ABI value
        jit_v = (0 if jit else -1) if isinstance(jit, bool) else int(jit)
        # wide_min: neurons of at least this many compartments run one per
        # warp (0: chosen by timing candidates at creation, negative: never)
        opt = GbhOptions(precision, steps_per_launch, warps_per_block, 1 if use_graph else 0, device, jit_v,
                         int(wide_min))
        err = GbhError()
        syn_p = C.byref(self.batch.syn) if self.batch.syn is not None else None
        if remote is None:
            h = self.lib.gbh_create(C.byref(self.batch.desc), syn_p, C.byref(opt), C.byref(err))
        else:
            self._remote = {k: np.ascontiguousarray(remote[k], dtype=t) for k, t in
                            (("src_start", np.int64), ("target_solver", np.int32), ("target_op", np.int32),
                             ("weight", np.float64), ("delay_steps", np.int32))}
            r = self._remote
            self.nremote = len(r["src_start"]) - 1
            rs = GbhRemoteSynapses(self.nremote, _ptr(r["src_start"], _lp), _ptr(r["target_solver"], _ip),
                                   _ptr(r["target_op"], _ip), _ptr(r["weight"], _dp), _ptr(r["delay_steps"], _ip),
                                   int(remote.get("first_solver", 0)))
            h = self.lib.gbh_create_dist(C.byref(self.batch.desc), syn_p, C.byref(rs), C.byref(opt), C.byref(err))
        if not h:
            raise EngineError(err)
        self.h = h

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("gbhsolve error %d: %s" % (rc, self.lib.gbh_last_error().decode()))

    def run(self, nsteps: int) -> None:
        self._check(self.lib.gbh_run(self.h, int(nsteps)))

    def run_noalloc(self, nsteps: int, stream_handle: int = 0) -> None:
        """gbh_run_noalloc: the step with the library's fixed flux scratch."""
        self._check(self.lib.gbh_run_noalloc(self.h, int(nsteps), C.c_void_p(stream_handle)))

    def run_async(self, nsteps: int, stream_handle: int) -> None:
        self._check(self.lib.gbh_run_async(self.h, int(nsteps), C.c_void_p(stream_handle)))

    def get_state(self):
        b = self.batch
        vm = np.empty_like(b.vm)
        chip = np.empty_like(b.chip)
        conc = np.array(b.conc, copy=True)
        ops = np.empty_like(b.ops)
        self._check(self.lib.gbh_get_state(self.h, _ptr(vm, _dp), _ptr(chip, _dp), _ptr(conc, _dp),
                                           _ptr(ops, _ip)))
        return dict(vm=b.split(vm, b.vm_start), chip=b.split(chip, b.chip_start),
                    conc=b.split(conc, b.conc_start), ops=b.split(ops, b.ops_start))

    def vm(self) -> np.ndarray:
        b = self.batch
        vm = np.empty_like(b.vm)
        self._check(self.lib.gbh_get_state(self.h, _ptr(vm, _dp), None, None, None))
        return vm

    def set_state(self, vm=None, chip=None, conc=None):
        b = self.batch
        args = []
        for arr, dt in ((vm, np.float64), (chip, np.float64), (conc, np.float64)):
            if arr is None:
                args.append(None)
            else:
                a = np.ascontiguousarray(np.concatenate(arr) if isinstance(arr, list) else arr, dtype=dt)
                self._tmp = getattr(self, "_tmp", []) + [a]
                args.append(_ptr(a, _dp))
        self._check(self.lib.gbh_set_state(self.h, *args))

    def enable_givals(self, on: bool = True):
        self._check(self.lib.gbh_enable_givals(self.h, 1 if on else 0))

    def givals(self):
        b = self.batch
        g = np.array(b.givals, copy=True)
        self._check(self.lib.gbh_get_givals(self.h, _ptr(g, _dp)))
        return b.split(g, b.givals_start)

    def itotal(self):
        """gbh_get_itotal: hsolve->itotal of every solver (empty for storemode 0)."""
        b = self.batch
        t = np.zeros(max(int(b.itotal_start[-1]), 1))
        self._check(self.lib.gbh_get_itotal(self.h, _ptr(t, _dp)))
        return b.split(t, b.itotal_start)

    def register_inputs(self, solver, chip_index, kind=None, sa=None, sb=None):
        """Inputs of h_in_msgs: kind IN_SET (chip[index] = v, the default),
        IN_ADD (chip[index] += v*sa*sb when v > 1e-10: SYN2 messages) or
        IN_FLUX (flux[index] = v, index a conc index)."""
        self._in_s = np.ascontiguousarray(solver, dtype=np.int32)
        self._in_c = np.ascontiguousarray(chip_index, dtype=np.int64)
        if kind is None and sa is None and sb is None:
            self._check(self.lib.gbh_register_inputs(self.h, len(self._in_s), _ptr(self._in_s, _ip),
                                                     _ptr(self._in_c, _lp)))
            return
        n = len(self._in_s)
        self._in_k = np.ascontiguousarray(kind if kind is not None else np.zeros(n), dtype=np.int32)
        self._in_a = np.ascontiguousarray(sa if sa is not None else np.ones(n), dtype=np.float64)
        self._in_b = np.ascontiguousarray(sb if sb is not None else np.ones(n), dtype=np.float64)
        self._check(self.lib.gbh_register_inputs_typed(self.h, n, _ptr(self._in_s, _ip), _ptr(self._in_k, _ip),
                                                       _ptr(self._in_c, _lp), _ptr(self._in_a, _dp),
                                                       _ptr(self._in_b, _dp)))

    def set_inputs_async(self, host_values: np.ndarray, stream_handle: int = 0):
        self._check(self.lib.gbh_set_inputs_async(self.h, _ptr(host_values, _dp), C.c_void_p(stream_handle)))

    def register_outputs(self, solver, row):
        self._out_s = np.ascontiguousarray(solver, dtype=np.int32)
        self._out_r = np.ascontiguousarray(row, dtype=np.int32)
        self._check(self.lib.gbh_register_outputs(self.h, len(self._out_s), _ptr(self._out_s, _ip),
                                                  _ptr(self._out_r, _ip)))

    def step_io(self, host_in, host_out, nsteps: int = 1, stream_handle: int = 0):
        """gbh_step_io: inputs, nsteps steps and outputs, copies pipelined
        (host_out complete after the second following call or io_sync)."""
        pin = _ptr(host_in, _dp) if host_in is not None else None
        pout = _ptr(host_out, _dp) if host_out is not None else None
        self._check(self.lib.gbh_step_io(self.h, pin, pout, int(nsteps), C.c_void_p(stream_handle)))

    def io_sync(self):
        self._check(self.lib.gbh_io_sync(self.h))

    def run_io(self, host_in, host_out, nsteps: int, block: int = 0, stream_handle: int = 0):
        """gbh_run_io: nsteps steps, row k of host_in (nsteps x n_in) applied
        before step k, row k of host_out (nsteps x n_out) read after it; the
        copies stream in blocks of `block` steps. Returns when host_out is
        complete."""
        for a, n in ((host_in, len(getattr(self, "_in_s", ()))), (host_out, len(getattr(self, "_out_s", ())))):
            if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous or a.size < nsteps * n):
                raise ValueError("run_io: arrays must be C-contiguous float64 with nsteps rows")
        pin = _ptr(host_in, _dp) if host_in is not None else None
        pout = _ptr(host_out, _dp) if host_out is not None else None
        self._check(self.lib.gbh_run_io(self.h, pin, pout, int(nsteps), int(block), C.c_void_p(stream_handle)))

    def get_outputs_async(self, host_values: np.ndarray, stream_handle: int = 0):
        self._check(self.lib.gbh_get_outputs_async(self.h, _ptr(host_values, _dp), C.c_void_p(stream_handle)))

    def loss_gradient(self, nsteps: int, solver, row, trace, checkpoint_every: int = 100):
        """gbh_loss_gradient: loss = sum over steps and targets of (Vm - trace)^2
        and its gradient with respect to chip[], ravals[] and the initial vm[]
        (flat arrays in the batch layout). The engine state is unchanged."""
        b = self.batch
        s = np.ascontiguousarray(solver, dtype=np.int32)
        r = np.ascontiguousarray(row, dtype=np.int32)
        tr = np.ascontiguousarray(trace, dtype=np.float64).reshape(int(nsteps), len(s))
        spec = GbhLossSpec(len(s), _ptr(s, _ip), _ptr(r, _ip), _ptr(tr, _dp))
        loss = C.c_double(0.0)
        dchip = np.zeros(int(b.chip_start[-1]) or 1)
        drav = np.zeros(int(b.ravals_start[-1]) or 1)
        dvm = np.zeros(int(b.vm_start[-1]) or 1)
        self._check(self.lib.gbh_loss_gradient(self.h, int(nsteps), int(checkpoint_every), C.byref(spec),
                                               C.byref(loss), _ptr(dchip, _dp), _ptr(drav, _dp), _ptr(dvm, _dp)))
        return loss.value, dchip, drav, dvm

    def get_spiked(self) -> np.ndarray:
        """gbh_get_spiked: bool per local solver, spiked since the last call."""
        n = self.batch.n
        bits = np.zeros((n + 7) // 8, dtype=np.uint8)
        self._check(self.lib.gbh_get_spiked(self.h, bits.ctypes.data_as(C.POINTER(C.c_uint8))))
        return np.unpackbits(bits, bitorder="little")[:n].astype(bool)

    def deliver_remote(self, spiked_sources) -> None:
        """gbh_deliver_remote: bool per remote source, spiked in the step just run."""
        bits = np.packbits(np.asarray(spiked_sources, dtype=bool), bitorder="little")
        bits = np.ascontiguousarray(bits, dtype=np.uint8)
        self._check(self.lib.gbh_deliver_remote(self.h, bits.ctypes.data_as(C.POINTER(C.c_uint8))))

    def spike_counts(self) -> np.ndarray:
        c = np.zeros(self.batch.n, dtype=np.int64)
        self._check(self.lib.gbh_get_spike_counts(self.h, _ptr(c, _lp)))
        return c

    def stats(self) -> GbhStats:
        st = GbhStats()
        self._check(self.lib.gbh_get_stats(self.h, C.byref(st)))
        return st

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
