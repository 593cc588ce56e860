"""Runs replayed from CUDA graphs (gbh_options.use_graph): the step number
lives on the device, so one captured graph serves every start step. Results
must equal plain launches bit for bit: spiking networks (event rings indexed
by the step), multi-step cable runs, calls of different lengths, graph and
plain calls interleaved on one engine, and the state sync in between."""
import numpy as np
import pytest

from gbhsolve import configs, model

pytestmark = pytest.mark.gpu


def _network(n, p, seed):
    rng = np.random.default_rng(seed)
    ms, syn = configs.hh_network(n, p_conn=p, seed=seed, delay=3e-4)
    for m, x in zip(ms, rng.uniform(0.0, 0.3e-9, size=n)):
        m.compartments[0].inject = x
    hs = [model.build(m) for m in ms]
    esyn, child = configs.network_synapses(hs, syn)
    return hs, esyn, child


@pytest.mark.parametrize("jit", [True, False])
def test_network_graph_matches_oracle(oracle, gpu_engine, jit):
    hs, esyn, child = _network(100, 0.08, seed=7)
    eng = gpu_engine.Engine(hs, synapses=esyn, jit=jit, use_graph=True)
    for n in (500, 500, 137, 863, 1000):   # repeated and odd lengths reuse / add graphs
        eng.run(n)
    solvers = [oracle.Solver(h, i) for i, h in enumerate(hs)]
    net = oracle.Network(solvers, esyn["src_start"], esyn["target_solver"], child, esyn["target_op"],
                         esyn["weight"], esyn["delay_steps"])
    net.run(3000)
    assert net.spikes.sum() > len(hs)
    np.testing.assert_array_equal(eng.spike_counts(), net.spikes)
    np.testing.assert_array_equal(eng.vm(), np.concatenate([s.vm for s in solvers]))
    assert eng.stats().steps == 3000
    eng.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_and_plain_interleaved(gpu_engine, precision):
    prec = gpu_engine.PREC_FP64 if precision == "fp64" else gpu_engine.PREC_MIXED
    hs, _ = configs.cables_replicated(200, gk_dend=36.0, seed=9)
    ref = gpu_engine.Engine(hs, precision=prec, steps_per_launch=16)
    g = gpu_engine.Engine(hs, precision=prec, steps_per_launch=16, use_graph=True)
    ref.run(1000)
    g.run(300)
    g.run(300)
    st = g.get_state()          # sync between replays
    g.set_state(vm=st["vm"], chip=st["chip"])
    g.run(400)
    np.testing.assert_array_equal(g.vm(), ref.vm())
    ref.close()
    g.close()


def test_network_graph_with_noalloc_between(oracle, gpu_engine):
    """A plain (no-allocation) run between graph replays leaves the device
    step counter stale; the next replay must resynchronise it."""
    hs, esyn, child = _network(60, 0.1, seed=11)
    eng = gpu_engine.Engine(hs, synapses=esyn, use_graph=True)
    eng.run(400)
    eng.run_noalloc(250)        # NULL stream: queued on the engine's own stream
    eng.run(350)
    solvers = [oracle.Solver(h, i) for i, h in enumerate(hs)]
    net = oracle.Network(solvers, esyn["src_start"], esyn["target_solver"], child, esyn["target_op"],
                         esyn["weight"], esyn["delay_steps"])
    net.run(1000)
    np.testing.assert_array_equal(eng.spike_counts(), net.spikes)
    np.testing.assert_array_equal(eng.vm(), np.concatenate([s.vm for s in solvers]))
    eng.close()
