"""Wide tiles: a neuron with many compartments runs on one thread block, its
compartments on separate threads, the elimination level by level. FP64
results equal the oracle (the reference's sequential step) bit for bit,
including the table bracket the reference carries from one compartment's
lookup to the next; wide_min=1 forces every eligible neuron wide so the
opcode, concentration and network programs run through the same kernel."""
import numpy as np
import pytest

import ophelpers as A
import test_conc_diffusion as CD
import opprograms as OP
from test_opcodes import FIXTURE, _compare
from gbhsolve import configs, model

pytestmark = pytest.mark.gpu


def _oracle_run(oracle, h, n):
    s = oracle.Solver(h)
    s.run(n)
    return s


@pytest.mark.parametrize("method", [model.BEULER, model.CRANK])
def test_random_trees_wide_fp64(oracle, gpu_engine, method):
    hs = [model.build(m) for m in configs.random_trees(24, size_range=(32, 200), seed=7, method=method)]
    eng = gpu_engine.Engine(hs, wide_min=32)
    assert eng.stats().tiles == len(hs)          # one neuron per tile: all wide
    eng.run(300)
    st = eng.get_state()
    for i in range(0, len(hs), 3):
        ref = _oracle_run(oracle, hs[i], 300)
        np.testing.assert_array_equal(st["vm"][i], ref.vm)
        np.testing.assert_array_equal(st["chip"][i], ref.chip)
        np.testing.assert_array_equal(st["conc"][i], ref.conc[:len(hs[i].conc)])
    eng.close()


def test_random_trees_wide_equals_lane(gpu_engine):
    """The same batch with and without wide tiles: bit-identical."""
    hs = [model.build(m) for m in configs.random_trees(40, size_range=(8, 120), seed=8)]
    a = gpu_engine.Engine(hs, wide_min=32)
    b = gpu_engine.Engine(hs, wide_min=-1)
    a.run(400)
    b.run(400)
    np.testing.assert_array_equal(a.vm(), b.vm())
    np.testing.assert_array_equal(a.get_state()["conc"][5], b.get_state()["conc"][5])
    a.close()
    b.close()


def test_random_trees_wide_mixed(oracle, gpu_engine):
    hs = [model.build(m) for m in configs.random_trees(16, size_range=(40, 160), seed=9)]
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_MIXED)
    refs = [oracle.Solver(h) for h in hs]
    worst = 0.0
    for _ in range(6):
        eng.run(500)
        for r in refs:
            r.run(500)
        worst = max(worst, float(np.max(np.abs(eng.vm() - np.concatenate([r.vm for r in refs])))))
    assert worst <= 1e-6, worst
    eng.close()


@pytest.mark.parametrize("name", sorted(OP.PROGRAMS))
def test_opcode_programs_forced_wide(oracle, gpu_engine, name):
    d = np.load(FIXTURE, allow_pickle=False)
    for mode in OP.MODES:
        tag = OP.mode_tag(name, *mode)
        h, libm = OP.from_fixture(d, tag), bool(d[tag + "/libm"])
        eng = gpu_engine.Engine([h], wide_min=1)
        eng.enable_givals(True)
        eng.run(OP.NSTEPS)
        st = eng.get_state()
        # the reference's own step code (fixture) and the oracle
        _compare(st["vm"][0], d[tag + "/vm"], libm, tag)
        _compare(st["chip"][0], d[tag + "/chip"], libm, tag)
        ref = _oracle_run(oracle, h, OP.NSTEPS)
        _compare(st["vm"][0], ref.vm, libm, tag)
        _compare(st["chip"][0], ref.chip, libm, tag)
        if len(h.conc):
            _compare(st["conc"][0], ref.conc[:len(h.conc)], libm, tag)
        _compare(eng.givals()[0], ref.givals, libm, tag)
        eng.close()


@pytest.mark.parametrize("name", sorted(CD.PROGRAMS))
def test_diffusion_programs_forced_wide(oracle, gpu_engine, name):
    h = CD.build(name)
    eng = gpu_engine.Engine([h], wide_min=1)
    eng.run(500)
    ref = _oracle_run(oracle, h, 500)
    st = eng.get_state()
    if name in CD.LIBM:
        np.testing.assert_allclose(st["conc"][0], ref.conc[:len(h.conc)], rtol=1e-11, atol=0)
        np.testing.assert_allclose(st["vm"][0], ref.vm, rtol=1e-11, atol=0)
    else:
        np.testing.assert_array_equal(st["conc"][0], ref.conc[:len(h.conc)])
        np.testing.assert_array_equal(st["vm"][0], ref.vm)
    eng.close()


def test_network_forced_wide(oracle, gpu_engine):
    """Spikegens and synchans in wide tiles: event delivery unchanged."""
    import test_network_parity as NP
    rng = np.random.default_rng(3)
    n = 60
    hs, esyn, child = NP._network(n, 0.1, seed=5, inject=rng.uniform(0.0, 0.3e-9, size=n))
    eng = gpu_engine.Engine(hs, synapses=esyn, wide_min=1)
    eng.run(2000)
    solvers, ref_spikes = NP._oracle_net(oracle, hs, esyn, child, 2000)
    assert ref_spikes.sum() > n
    np.testing.assert_array_equal(eng.spike_counts(), ref_spikes)
    np.testing.assert_array_equal(eng.vm(), np.concatenate([s.vm for s in solvers]))
    eng.close()


def _bracket_edge(h):
    """A table row r whose lower edge xvals[r] floors to row r-1 when looked
    up fresh ((x - xmin) * invdx rounds below r), or None."""
    xv = np.asarray(h.xvals)
    for r in range(1, h.xdivs):
        x = float(xv[r])
        if int((x - h.xmin) * h.invdx) == r - 1:
            return r, x
    return None


def test_table_bracket_carried_between_compartments(oracle, gpu_engine):
    """The reference keeps the previous compartment's table bracket while Vm
    stays inside it (hines_chip.c:174-203). With compartment k at a Vm inside
    row r and compartment k+1 exactly at xvals[r] (which a fresh lookup puts
    in row r-1), the cached bracket wins: the wide kernel must replay the
    chain, and still equal the oracle bit for bit."""
    m = configs.cables(1, ncomp=48, gk_dend=36.0)[0]
    h = model.build(m)
    edge = _bracket_edge(h)
    if edge is None:
        pytest.skip("no rounding edge in this table")
    r, x = edge
    dx = 1.0 / h.invdx
    vm = np.array(h.vm, copy=True)
    vm[10] = x + 0.3 * dx     # inside row r
    vm[11] = x                # the edge: cached row r, fresh row r - 1
    vm[30] = x + 0.6 * dx
    vm[31] = x
    h.vm = vm
    eng = gpu_engine.Engine([h], wide_min=32)
    assert eng.stats().tiles == 1
    ref = oracle.Solver(h)
    for _ in range(3):
        eng.run(1)
        ref.run(1)
        st = eng.get_state()
        np.testing.assert_array_equal(st["vm"][0], ref.vm)
        np.testing.assert_array_equal(st["chip"][0], ref.chip)
    eng.close()
