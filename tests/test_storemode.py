"""storemode: hsolve->itotal, the per-step sum over a solver of its leak
currents and STORE_ALLI_OP channel currents (storemode 1) or STORE_ALLC_OP
channel conductances (storemode 2), hines_chip.c:134-166, 314-322.

* CPU: the oracle against the reference's own step code (where its sources
  are present); the decoder's checks (a STORE op needs storemode, its index
  must lie in itotal; a storemode solver of several trees is one neuron).
* GPU: the engine against the oracle, bit for bit in FP64 (vm, chip, itotal)
  for storemode 1 and 2, single- and multi-tree solvers, batched with
  storemode-0 solvers; mixed precision within tolerance.
"""
import os

import numpy as np
import pytest

import ophelpers as A

STORE_ALLI, STORE_ALLC = 3501, 3502
DT = 2e-5
NELM = 5


def _c(vm0=-0.062, inj=1e-10):
    return A.Compt(-0.065 / 3e8, inj, DT / 1e-11, 1.0 + DT / (1e-11 * 3e8), 3e8, vm0)


def _solver(mode, parents, seed=0, pump=True, crank=False):
    """Compartments with two HH-like channels each (and a pump on the first
    row), a STORE op after every channel when mode > 0."""
    rng = np.random.default_rng(seed)
    store = STORE_ALLI if mode == 1 else STORE_ALLC
    compts = []
    for r in range(len(parents)):
        c = _c(-0.062 + 0.004 * rng.random(), (1 + 3 * rng.random()) * 1e-10)
        if pump and r == 0:
            c.op(A.CONC_VAL, 0).op(A.ELMMPUMP, chips=[2e-4, 3e-12, 1e-3], giv=1)
            if mode == 1:
                c.op(STORE_ALLI, 4)
        c.op(A.NEWVOLT).op(A.CHAN_EK, chips=[0.05, (1 + rng.random()) * 1e-8]).op(A.IPOL1V, 0, 3, chips=[0.1])
        c.op(A.IPOL1V, 2, 1, chips=[0.6]).op(A.ADD_CURR, giv=3)
        if mode:
            c.op(store, 1 + (r % 2))
        c.op(A.CHAN_EK, chips=[-0.08, (2 + rng.random()) * 1e-8]).op(A.IPOL1V, 4, 4, chips=[0.3]).op(A.ADD_CURR, giv=3)
        if mode:
            c.op(store, 3)
        compts.append(c)
    h = A.solver(compts, A.tables(12, 40, seed=seed), dt=DT, conc=[1e-4] if pump else (), parents=parents,
                 crank=crank)
    h.storemode = mode
    h.nelm_names = NELM if mode else 0
    return h


CHAIN = [1, 2, -1]
TWO_TREES = [1, -1, 3, 4, -1]


def test_decoder_needs_storemode_for_store_ops():
    from gbhsolve import engine
    h = _solver(1, CHAIN)
    h.storemode = 0
    with pytest.raises(engine.EngineError) as ei:
        engine.validate([h])
    assert ei.value.code == -1 and ei.value.opcode == STORE_ALLI


def test_decoder_checks_itotal_index():
    from gbhsolve import engine
    h = _solver(2, CHAIN)
    h.nelm_names = 3          # the program stores into itotal[3]
    with pytest.raises(engine.EngineError) as ei:
        engine.validate([h])
    assert ei.value.code == -1 and ei.value.opcode == STORE_ALLC


def test_storemode_solver_is_one_neuron():
    from gbhsolve import engine
    assert engine.validate([_solver(0, TWO_TREES)])[0] == 2
    assert engine.validate([_solver(1, TWO_TREES)])[0] == 1


needs_ref = pytest.mark.skipif(
    not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref", "libhsolve_ref.so")),
    reason="the reference's step code is built only where its sources are present")


@needs_ref
@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("parents", [CHAIN, TWO_TREES])
def test_oracle_matches_reference(oracle, mode, parents):
    h = _solver(mode, parents, seed=3)
    a, b = oracle.Solver(h), oracle.Solver(h)
    a.run(300, "oracle")
    b.run(300, "reference")
    np.testing.assert_array_equal(a.vm, b.vm)
    np.testing.assert_array_equal(a.chip, b.chip)
    np.testing.assert_array_equal(a.itotal, b.itotal)
    assert np.count_nonzero(a.itotal) == (5 if mode == 1 else 3)


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [True, False])
@pytest.mark.parametrize("crank", [False, True])
def test_engine_fp64_bitwise(oracle, gpu_engine, jit, crank):
    hs = []
    for k in range(6):
        hs.append(_solver(k % 3, TWO_TREES if k % 2 else CHAIN, seed=k, crank=crank))
    eng = gpu_engine.Engine(hs * 3, jit=jit, steps_per_launch=23)
    assert all(not np.any(t) for t in eng.itotal())   # no step run yet
    eng.run(250)
    st = eng.get_state()
    it = eng.itotal()
    for i, h in enumerate(hs * 3):
        ref = oracle.Solver(h)
        ref.run(250)
        np.testing.assert_array_equal(st["vm"][i], ref.vm, err_msg=str(i))
        np.testing.assert_array_equal(st["chip"][i], ref.chip, err_msg=str(i))
        if h.storemode:
            np.testing.assert_array_equal(it[i], ref.itotal, err_msg=str(i))
        else:
            assert len(it[i]) == 0
    eng.close()


@pytest.mark.gpu
def test_engine_mixed_within_tolerance(oracle, gpu_engine):
    hs = [_solver(1, CHAIN, seed=7), _solver(2, TWO_TREES, seed=8)]
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_MIXED)   # autotuned: trial steps run here
    assert all(not np.any(t) for t in eng.itotal())
    eng.run(300)
    it = eng.itotal()
    vm = eng.get_state()["vm"]
    for i, h in enumerate(hs):
        ref = oracle.Solver(h)
        ref.run(300)
        np.testing.assert_allclose(vm[i], ref.vm, rtol=0, atol=1e-9)
        np.testing.assert_allclose(it[i], ref.itotal, rtol=1e-6, atol=1e-6 * np.max(np.abs(ref.itotal)))
    eng.close()


def test_storemode_types_are_not_specialised():
    """storemode solvers run on the interpreting kernels: the code generator
    declines their tile type (empty source), as it does for symmetric
    compartments."""
    from gbhsolve import engine
    assert engine.jit_source([_solver(1, CHAIN)]) == ""
    assert engine.jit_source([_solver(0, CHAIN)]) != ""
