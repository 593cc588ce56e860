"""The hsolve-level ABI (include/gbh_hsolve.h): GENESIS solvers registered
one by one, each called once per step in the scheduler's order, stepped
together by one batch engine -- the one-hsolve-per-cell idiom the reference
batches in its CUDA backend (genesis/src/hines/cuda/cuda_hsolve.c:64-145).

* 64 per-cell hsolves with spike detectors and synchans: synapses go to the
  device, the first call of a step runs the whole batch in one kernel launch,
  and Vm and spike counts equal the CPU oracle's network bit for bit; host
  spike callbacks fire once per spike.
* Per-cell random trees with Ca pools, inject inputs read through message
  value callbacks every step, Vm written back every step (h_out_msgs), and
  a state sync / host edit / push in the middle of the run: bit-exact
  against the oracle stepping the same inputs.
"""
import numpy as np
import pytest

from gbhsolve import configs, model

pytestmark = pytest.mark.gpu
IN_SET = 0


@pytest.fixture
def hs_api(gpu_engine):
    from gbhsolve import hsolve
    hsolve.cleanup()
    yield hsolve
    hsolve.cleanup()


def test_network_of_per_cell_hsolves(oracle, hs_api):
    n = 64
    ms, syn = configs.hh_network(n, p_conn=0.15, seed=21)
    rng = np.random.default_rng(22)
    inj = rng.uniform(0.0, 0.3e-9, size=n)
    hs = [model.build(m) for m in ms]
    esyn, child = configs.network_synapses(hs, syn)
    w = rng.uniform(0.5, 1.5, size=len(esyn["weight"])).astype(np.float32).astype(np.float64)
    d = rng.integers(1, 4, size=len(w)).astype(np.int32)
    # inject arrives as an INJECT message each step (a value callback)
    inject_row = [int(h.compchips[0]) + 1 for h in hs]
    host_spikes = np.zeros(n, dtype=np.int64)
    solvers = []
    for i, h in enumerate(hs):
        lo, hi = esyn["src_start"][i], esyn["src_start"][i + 1]
        synapses = [(int(esyn["target_solver"][k]), int(esyn["target_op"][k]), float(w[k]), int(d[k]))
                    for k in range(lo, hi)]

        def bump(i=i):
            host_spikes[i] += 1

        s = hs_api.Solver(h, inputs=[(IN_SET, inject_row[i], 1.0, 1.0, lambda x=float(inj[i]): x)],
                          synapses=synapses, on_spike=bump)
        solvers.append(s)
    for s in solvers:
        s.register()
    nsteps = 1500
    for step in range(nsteps):
        for s in solvers:          # the scheduler calls every hsolve once per step
            assert s.step(step) == 1
    st = hs_api.stats()
    assert st.steps == nsteps
    assert st.launches == nsteps          # one launch per step for all 64 solvers
    for s in solvers:
        s.sync()
    # the oracle network with the same inputs, weights and delays
    sv = []
    for i, h in enumerate(hs):
        o = oracle.Solver(h, i)
        o.chip[inject_row[i]] = float(inj[i])
        sv.append(o)
    net = oracle.Network(sv, esyn["src_start"], esyn["target_solver"], child, esyn["target_op"], w, d)
    net.run(nsteps)
    assert net.spikes.sum() > n
    np.testing.assert_array_equal(host_spikes, net.spikes)
    for s, o in zip(solvers, sv):
        np.testing.assert_array_equal(s.vm, o.vm)


def test_trees_inputs_outputs_sync_push(oracle, hs_api):
    hs = [model.build(m) for m in configs.random_trees(24, size_range=(8, 64), seed=23)]
    rng = np.random.default_rng(24)
    inj = rng.uniform(0.0, 1e-9, size=(len(hs), 300))
    clock = {"step": 0}
    solvers = []
    for i, h in enumerate(hs):
        row = int(h.compchips[h.ncompts - 1]) + 1        # the soma's inject (the root is the last row)
        s = hs_api.Solver(h, inputs=[(IN_SET, row, 1.0, 1.0, lambda i=i: inj[i, clock["step"]])],
                          has_outputs=(i % 3 == 0))
        s.row = row
        solvers.append(s)
    for s in solvers:
        s.register()
    orc = [oracle.Solver(h) for h in hs]
    for step in range(300):
        clock["step"] = step
        for i, s in enumerate(solvers):
            s.step(step)
        for i, o in enumerate(orc):
            o.chip[solvers[i].row] = inj[i, step]
            o.run(1)
        for i, s in enumerate(solvers):
            if i % 3 == 0:                       # written back every step for h_out_msgs
                np.testing.assert_array_equal(s.vm, orc[i].vm)
        if step == 150:                          # RESTORE2-style edit of one solver's state
            solvers[5].sync()
            np.testing.assert_array_equal(solvers[5].chip, orc[5].chip)
            solvers[5].vm[:] += 1e-3
            orc[5].vm[:] += 1e-3
            solvers[5].push()
    for i, s in enumerate(solvers):
        s.sync()
        np.testing.assert_array_equal(s.vm, orc[i].vm)
        np.testing.assert_array_equal(s.conc, orc[i].conc[:len(s.conc)])
