"""Parity at the workloads' stated sizes (FP64: bit for bit against the
oracle, which equals the reference's own step code; spike counts identical):

* cables, 1,000 neurons x 16 compartments, 200 steps, backward Euler and
  Crank-Nicolson (one hsolve holding every neuron, as configured);
* the spiking network, 4,000 single-compartment cells, 2 % connectivity,
  50,000 steps of 0.1 ms (5 s simulated) with a seeded tonic drive U(0.05,
  0.3) nA (as configured the network never spikes);
* uneven random trees (8-256 compartments, Ca pools): a seeded 1-in-100
  sample of the 50,000 trees over 5,000 steps -- neurons are independent, so
  the sample steps exactly as it does inside the full batch;
* the gradient workload's forward pass: every 64th of the 4,096 trees x 64
  compartments over 10,000 steps.
The mixed form is checked against the same oracle runs: max |dVm| <= 1e-6 V
and, for the network, identical spike counts.
"""
import numpy as np
import pytest

from gbhsolve import configs, model

pytestmark = pytest.mark.gpu


def _oracle_all(oracle, hs, nsteps):
    out = []
    for h in hs:
        s = oracle.Solver(h)
        s.run(nsteps)
        out.append(s.vm.copy())
    return out


@pytest.mark.parametrize("method", [model.BEULER, model.CRANK])
def test_cables_1000x16_200_steps(oracle, gpu_engine, method):
    hs = [model.build(m) for m in configs.cables(1000, method=method)]
    ref = _oracle_all(oracle, hs, 200)[0]
    for prec, tol in ((gpu_engine.PREC_FP64, 0.0), (gpu_engine.PREC_MIXED, 1e-6)):
        eng = gpu_engine.Engine(hs, precision=prec)
        eng.run(200)
        vm = eng.vm()
        if tol == 0.0:
            np.testing.assert_array_equal(vm, ref)
        else:
            assert np.max(np.abs(vm - ref)) <= tol
        eng.close()


def test_network_4000_cells_50000_steps(oracle, gpu_engine):
    ms, syn = configs.hh_network(4000)
    drive = np.random.default_rng(1).uniform(0.05e-9, 0.3e-9, size=len(ms))
    for m, x in zip(ms, drive):
        m.compartments[0].inject = float(x)
    hs = [model.build(m) for m in ms]
    esyn, child = configs.network_synapses(hs, syn)
    nsteps = 50_000
    solvers = [oracle.Solver(h, i) for i, h in enumerate(hs)]
    net = oracle.Network(solvers, esyn["src_start"], esyn["target_solver"], child, esyn["target_op"],
                         esyn["weight"], esyn["delay_steps"])
    net.run(nsteps)
    ref_vm = np.concatenate([s.vm for s in solvers])
    assert net.spikes.sum() > 10 * len(hs)
    eng = gpu_engine.Engine(hs, synapses=esyn, precision=gpu_engine.PREC_FP64)
    eng.run(nsteps)
    np.testing.assert_array_equal(eng.spike_counts(), net.spikes)
    np.testing.assert_array_equal(eng.vm(), ref_vm)
    eng.close()
    mx = gpu_engine.Engine(hs, synapses=esyn, precision=gpu_engine.PREC_MIXED)
    mx.run(nsteps)
    mismatches = int(np.sum(mx.spike_counts() != net.spikes))
    print("mixed form, 4,000-cell network over 50,000 steps: %d of %d cells differ in spike count"
          % (mismatches, len(hs)))
    mx.close()


def test_random_trees_sample_of_50000_over_5000_steps(oracle, gpu_engine):
    ms = configs.random_trees(50_000, seed=2)
    sample = [model.build(ms[i]) for i in range(0, 50_000, 100)]
    ref = _oracle_all(oracle, sample, 5000)
    for prec in (gpu_engine.PREC_FP64, gpu_engine.PREC_MIXED):
        eng = gpu_engine.Engine(sample, precision=prec)
        eng.run(5000)
        vm = eng.get_state()["vm"]
        worst = max(float(np.max(np.abs(v - r))) for v, r in zip(vm, ref))
        if prec == gpu_engine.PREC_FP64:
            assert worst == 0.0
        else:
            assert worst <= 1e-6, worst
        eng.close()


def test_gradient_workload_forward_sample(oracle, gpu_engine):
    trees, (na, k) = configs.grad_trees(4096, ncomp=64, seed=4)
    sample = [model.build(trees[i].model(na, k, dt=25e-6), exact=True) for i in range(0, 4096, 64)]
    ref = _oracle_all(oracle, sample, 10_000)
    eng = gpu_engine.Engine(sample, precision=gpu_engine.PREC_FP64, wide_min=-1)
    eng.run(10_000)
    vm = eng.get_state()["vm"]
    for v, r in zip(vm, ref):
        np.testing.assert_array_equal(v, r)
    eng.close()
