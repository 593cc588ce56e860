"""gbh_run_noalloc: the step entry point that allocates no device memory.

It is for hosts that may not allocate device memory while stepping: the
GPU's memory was reserved at start-up by a pool another runtime owns, or
the step loop cannot afford cudaMalloc/cudaFree, which may synchronise the
whole device. Its Ca-flux scratch is a fixed array inside the library, so
these tests use models with Ca pools, where that scratch is really used, and
check consecutive calls against gbh_run on an identical engine. The FP64
step is exact, so every comparison is bit for bit, the tolerance the other
FP64 engine tests use. Calls with a NULL stream run on the engine's own
stream, so no device-wide synchronisation stands between a call and the
state read that follows it. This file is collected last on purpose.
"""
import numpy as np
import pytest

from gbhsolve import configs, model
import ophelpers as A

pytestmark = pytest.mark.gpu
DT = 2e-5
GBH_ERR_ARG = -1
FLUX_MAX = 1 << 20


def _assert_same(a, b, n):
    for i in range(n):
        np.testing.assert_array_equal(b["vm"][i], a["vm"][i])
        np.testing.assert_array_equal(b["conc"][i], a["conc"][i])
        np.testing.assert_array_equal(b["chip"][i], a["chip"][i])


def _flux_model(nshells=4, seed=5):
    """One compartment feeding a Ca diffusion system: a Ca channel's current
    goes into shell 0 through FLUX_OP, a FLUX message sets shell 2's flux."""
    rng = np.random.default_rng(seed)
    cov0, _, conc = A.diffusion_system(rng, nshells, dt=DT, crank=True)
    c = A.Compt(emrm=-0.065 / 1e9, inject=1e-10, tbyc=DT / 1e-11, diag=1.0 + DT / 1e-11 / 1e9, rm=1e9, vm0=-0.06)
    c.op(A.NEWVOLT).op(A.CONC_VAL, 0).op(A.CHAN_EK, chips=[0.12, 3e-11]).op(A.IPOL1V, 0, 4, chips=[0.3])
    c.op(A.ADD_CURR, giv=3).op(A.FLUX)
    ops = [A.FCONC, 0, A.FLUXCONC, A.CONC, 2, A.FLUXCONC, A.MMPUMP, A.LCONC]
    chips = [0.0, 5e5, 1e-9, 2e5, 1e-6, 1e-3]
    diff = dict(dconc=[0], nshells=[nshells], nshrows=[1], nshfix=[0], fbufval=[0], covals0=cov0, bufvals=[])
    return A.solver([c], A.tables(12, 40, seed=3), dt=DT, crank=True, conc=conc, concops=ops, concchip=chips,
                    diff=diff)


def _inputs(eng, gpu_engine):
    # inject (set) and a flux message into shell 2 (set)
    kinds = np.array([gpu_engine.IN_SET, gpu_engine.IN_FLUX])
    eng.register_inputs(np.zeros(2, np.int32), np.array([1, 2]), kind=kinds)


def test_run_noalloc_matches_run_twice(gpu_engine):
    hs = [model.build(m) for m in configs.random_trees(40, size_range=(8, 48), seed=11)]
    ref = gpu_engine.Engine(hs, steps_per_launch=25)
    new = gpu_engine.Engine(hs, steps_per_launch=25)
    for _ in range(2):
        ref.run(120)
        new.run_noalloc(120)          # NULL stream: the engine's own stream
        _assert_same(ref.get_state(), new.get_state(), len(hs))
    assert new.stats().steps == 240
    ref.close()
    new.close()


def test_run_noalloc_keeps_flux_inputs(gpu_engine):
    """FLUX and SET inputs placed by gbh_set_inputs_async before each call are
    stepped on exactly as gbh_run steps on them, with gbh_run and
    gbh_run_noalloc calls interleaved on one engine."""
    h = _flux_model()
    ref = gpu_engine.Engine([h], steps_per_launch=1)
    new = gpu_engine.Engine([h], steps_per_launch=1)
    _inputs(ref, gpu_engine)
    _inputs(new, gpu_engine)
    rng = np.random.default_rng(21)
    for k in range(120):
        v = np.array([rng.uniform(0, 3e-10), rng.uniform(-1e-13, 1e-12)])
        ref.set_inputs_async(v, 0)
        new.set_inputs_async(v, 0)
        ref.run(1)
        if k % 3 == 2:
            new.run(1)
        else:
            new.run_noalloc(1)
        if k % 40 == 39:
            _assert_same(ref.get_state(), new.get_state(), 1)
    assert np.any(ref.get_state()["conc"][0] != h.conc)
    ref.close()
    new.close()


def test_run_noalloc_on_a_caller_stream(gpu_engine):
    """Inputs and steps queued on the caller's stream run in that order; the
    caller waits for its own stream before reading the state."""
    import torch
    h = _flux_model()
    ref = gpu_engine.Engine([h], steps_per_launch=1)
    new = gpu_engine.Engine([h], steps_per_launch=1)
    _inputs(ref, gpu_engine)
    _inputs(new, gpu_engine)
    s = torch.cuda.Stream()
    rng = np.random.default_rng(22)
    for _ in range(2):
        v = np.array([rng.uniform(0, 3e-10), rng.uniform(0, 1e-12)])
        ref.set_inputs_async(v, 0)
        ref.run(30)
        new.set_inputs_async(v, s.cuda_stream)
        new.run_noalloc(30, s.cuda_stream)
        s.synchronize()
        _assert_same(ref.get_state(), new.get_state(), 1)
    ref.close()
    new.close()


def test_run_noalloc_allocates_nothing(gpu_engine):
    """Free device memory is the same before and after calls (the first call,
    which may load the library's device image, is made before measuring)."""
    import torch
    hs = [model.build(m) for m in configs.random_trees(40, size_range=(8, 48), seed=12)]
    eng = gpu_engine.Engine(hs, steps_per_launch=10)
    eng.run_noalloc(10)
    eng.vm()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        eng.run_noalloc(50)
    eng.vm()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    eng.close()


def test_run_noalloc_rejects_an_oversize_engine(gpu_engine):
    """An engine whose flux rows exceed the fixed array is refused before any
    work is queued; its state stays as it was."""
    h = _flux_model(nshells=FLUX_MAX // 32 + 8)
    eng = gpu_engine.Engine([h], steps_per_launch=1)
    before = eng.get_state()
    rc = eng.lib.gbh_run_noalloc(eng.h, 5, None)
    assert rc == GBH_ERR_ARG
    _assert_same(before, eng.get_state(), 1)
    assert eng.stats().steps == 0
    eng.close()


def test_run_noalloc_large_engine_then_small(gpu_engine):
    """A large engine fills most of the shared array; a small engine stepped
    after it must not see the large one's flux rows."""
    big = _flux_model(nshells=FLUX_MAX // 32 - 64, seed=6)
    eb_ref = gpu_engine.Engine([big], steps_per_launch=1)
    eb = gpu_engine.Engine([big], steps_per_launch=1)
    eb_ref.run(3)
    eb.run_noalloc(3)
    _assert_same(eb_ref.get_state(), eb.get_state(), 1)
    h = _flux_model()
    ref = gpu_engine.Engine([h], steps_per_launch=1)
    new = gpu_engine.Engine([h], steps_per_launch=1)
    for _ in range(2):
        ref.run(40)
        new.run_noalloc(40)
        _assert_same(ref.get_state(), new.get_state(), 1)
    for e in (eb_ref, eb, ref, new):
        e.close()
