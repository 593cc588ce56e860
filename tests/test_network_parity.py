"""Spiking network (one hsolve per cell, spikegen -> synchan events): the
GPU engine's device-side event delivery against the CPU oracle's restatement
of the synchan event queue. FP64: Vm bit for bit and identical spike counts."""
import numpy as np
import pytest

from gbhsolve import configs, model

pytestmark = pytest.mark.gpu


def _network(n, p, seed, delay=1e-4, weight=1.0, inject=None):
    ms, syn = configs.hh_network(n, p_conn=p, seed=seed, delay=delay, weight=weight)
    if inject is not None:
        for m, x in zip(ms, inject):
            m.compartments[0].inject = x
    hs = [model.build(m) for m in ms]
    esyn, child = configs.network_synapses(hs, syn)
    return hs, esyn, child


def _oracle_net(oracle, hs, esyn, child, nsteps):
    solvers = [oracle.Solver(h, i) for i, h in enumerate(hs)]
    net = oracle.Network(solvers, esyn["src_start"], esyn["target_solver"], child, esyn["target_op"],
                         esyn["weight"], esyn["delay_steps"])
    net.run(nsteps)
    return solvers, net.spikes


@pytest.mark.parametrize("jit", [True, False, 2, 3])
def test_network_spikes_and_vm_bitwise(oracle, gpu_engine, jit):
    rng = np.random.default_rng(3)
    n = 120
    inj = rng.uniform(0.0, 0.3e-9, size=n)
    hs, esyn, child = _network(n, 0.08, seed=5, inject=inj)
    eng = gpu_engine.Engine(hs, synapses=esyn, jit=jit)
    eng.run(3000)
    spikes = eng.spike_counts()
    vm = eng.vm()
    solvers, ref_spikes = _oracle_net(oracle, hs, esyn, child, 3000)
    assert ref_spikes.sum() > n      # the network is active
    np.testing.assert_array_equal(spikes, ref_spikes)
    np.testing.assert_array_equal(vm, np.concatenate([s.vm for s in solvers]))


def test_network_longer_delays(oracle, gpu_engine):
    rng = np.random.default_rng(4)
    n = 60
    hs, esyn, child = _network(n, 0.15, seed=6, delay=7.3e-4, inject=rng.uniform(0.05e-9, 0.25e-9, n))
    assert esyn["delay_steps"].max() >= 7
    eng = gpu_engine.Engine(hs, synapses=esyn)
    eng.run(2500)
    solvers, ref_spikes = _oracle_net(oracle, hs, esyn, child, 2500)
    np.testing.assert_array_equal(eng.spike_counts(), ref_spikes)
    np.testing.assert_array_equal(eng.vm(), np.concatenate([s.vm for s in solvers]))


@pytest.mark.parametrize("K", [1, 16, 50])
def test_network_cooperative_launches(oracle, gpu_engine, K):
    """K steps per cooperative launch with a grid barrier between steps equal
    the oracle bit for bit (calls of odd lengths split the K-step chunks)."""
    rng = np.random.default_rng(8)
    n = 150
    hs, esyn, child = _network(n, 0.07, seed=9, inject=rng.uniform(0.0, 0.3e-9, size=n))
    eng = gpu_engine.Engine(hs, synapses=esyn, steps_per_launch=-K)
    assert eng.stats().cooperative == 1
    for m in (700, 333, 967):
        eng.run(m)
    solvers, ref_spikes = _oracle_net(oracle, hs, esyn, child, 2000)
    assert ref_spikes.sum() > n
    np.testing.assert_array_equal(eng.spike_counts(), ref_spikes)
    np.testing.assert_array_equal(eng.vm(), np.concatenate([s.vm for s in solvers]))
    eng.close()


def test_network_cooperative_mixed_matches_launches(gpu_engine):
    """Mixed form: the cooperative plan equals per-step launches of the same
    interpreting kernel bit for bit."""
    rng = np.random.default_rng(10)
    n = 120
    hs, esyn, _ = _network(n, 0.08, seed=10, inject=rng.uniform(0.0, 0.3e-9, size=n))
    a = gpu_engine.Engine(hs, synapses=esyn, precision=gpu_engine.PREC_MIXED, jit=False, steps_per_launch=1)
    b = gpu_engine.Engine(hs, synapses=esyn, precision=gpu_engine.PREC_MIXED, jit=False, steps_per_launch=-32)
    a.run(1500)
    b.run(1500)
    np.testing.assert_array_equal(a.spike_counts(), b.spike_counts())
    np.testing.assert_array_equal(a.vm(), b.vm())
    assert a.spike_counts().sum() > n
    a.close()
    b.close()


def _weighted(esyn, seed, zero_frac=0.3, max_delay=6):
    """Seeded weights per synapse (a float field in the reference, so rounded
    through float) and delays of 0..max_delay steps, a share of them 0
    (a synapse delay under a tenth of a step)."""
    rng = np.random.default_rng(seed)
    n = len(esyn["weight"])
    w = rng.uniform(0.2, 2.0, size=n).astype(np.float32).astype(np.float64)
    d = rng.integers(1, max_delay + 1, size=n)
    d[rng.random(n) < zero_frac] = 0
    out = dict(esyn)
    out["weight"] = w
    out["delay_steps"] = d.astype(np.int32)
    return out


@pytest.mark.parametrize("jit", [True, False])
def test_network_weights_per_synapse_and_zero_delays(oracle, gpu_engine, jit):
    """Every synapse its own weight, some acting in the step of the spike:
    activations summed newest first as the reference's pending list does;
    identical spike counts and Vm bit for bit."""
    rng = np.random.default_rng(12)
    n = 150
    hs, esyn, child = _network(n, 0.08, seed=13, inject=rng.uniform(0.0, 0.3e-9, size=n))
    ws = _weighted(esyn, 14)
    assert (ws["delay_steps"] == 0).any() and len(np.unique(ws["weight"])) > 100
    eng = gpu_engine.Engine(hs, synapses=ws, jit=jit)
    for m in (1000, 777, 1223):
        eng.run(m)
    solvers, ref_spikes = _oracle_net(oracle, hs, ws, child, 3000)
    assert ref_spikes.sum() > n
    np.testing.assert_array_equal(eng.spike_counts(), ref_spikes)
    np.testing.assert_array_equal(eng.vm(), np.concatenate([s.vm for s in solvers]))
    eng.close()


def test_network_weights_graph_replay(oracle, gpu_engine):
    rng = np.random.default_rng(15)
    n = 100
    hs, esyn, child = _network(n, 0.1, seed=16, inject=rng.uniform(0.0, 0.3e-9, size=n))
    ws = _weighted(esyn, 17, zero_frac=0.5, max_delay=3)
    eng = gpu_engine.Engine(hs, synapses=ws, use_graph=True)
    for _ in range(4):
        eng.run(500)
    solvers, ref_spikes = _oracle_net(oracle, hs, ws, child, 2000)
    np.testing.assert_array_equal(eng.spike_counts(), ref_spikes)
    np.testing.assert_array_equal(eng.vm(), np.concatenate([s.vm for s in solvers]))
    eng.close()
