"""Partitioned spiking networks (one engine per rank, spikes all-gathered
every step and delivered into the targets' event rings).

* The partitioning and the exchange's timing rules on CPU: ranks simulated by
  the oracle's network layer with events delivered from the other ranks'
  spikes, in one process and as two gloo processes, equal the single-process
  oracle network bit for bit (Vm and spike counts).
* The engine's side (gbh_create_dist, gbh_get_spiked, gbh_deliver_remote):
  two engines in one process standing in for two ranks equal the oracle.
"""
import os
import sys

import numpy as np
import pytest

from gbhsolve import configs, model, shard
from oracle_rank import OracleRank

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _network(n, p, seed, delay=3e-4):
    rng = np.random.default_rng(seed)
    ms, syn = configs.hh_network(n, p_conn=p, seed=seed, delay=delay)
    for m, x in zip(ms, rng.uniform(0.0, 0.3e-9, size=n)):
        m.compartments[0].inject = x
    hs = [model.build(m) for m in ms]
    esyn, child = configs.network_synapses(hs, syn)
    return hs, esyn, child


def _oracle_whole(oracle, hs, esyn, child, nsteps):
    sol = [oracle.Solver(h, i) for i, h in enumerate(hs)]
    net = oracle.Network(sol, esyn["src_start"], esyn["target_solver"], child, esyn["target_op"], esyn["weight"],
                         esyn["delay_steps"])
    net.run(nsteps)
    return np.concatenate([s.vm for s in sol]), net.spikes.copy()


def test_partition_tables():
    hs, esyn, child = _network(40, 0.2, seed=3)
    n = len(hs)
    total = 0
    for r in range(3):
        lo, hi = shard.shard_range(n, r, 3)
        loc, rem = shard.partition_network(esyn, lo, hi, target_child=child)
        assert len(loc["src_start"]) == hi - lo + 1 and len(rem["src_start"]) == n + 1
        for s in range(lo, hi):            # local sources have no remote synapses
            assert rem["src_start"][s] == rem["src_start"][s + 1]
        assert np.all((loc["target_solver"] >= 0) & (loc["target_solver"] < hi - lo))
        assert np.all((rem["target_solver"] >= 0) & (rem["target_solver"] < hi - lo))
        total += len(loc["weight"]) + len(rem["weight"])
    assert total == len(esyn["weight"])      # every synapse lands on exactly one rank


@pytest.mark.parametrize("world", [2, 3])
def test_partitioned_oracle_in_process(oracle, world):
    hs, esyn, child = _network(60, 0.1, seed=5)
    n, nsteps = len(hs), 800
    ref_vm, ref_sp = _oracle_whole(oracle, hs, esyn, child, nsteps)
    assert ref_sp.sum() > n
    ranks = []
    for r in range(world):
        lo, hi = shard.shard_range(n, r, world)
        loc, rem = shard.partition_network(esyn, lo, hi, target_child=child)
        ranks.append(OracleRank(oracle, hs[lo:hi], loc, rem))
    for _ in range(nsteps):
        for rk in ranks:
            rk.run(1)
        glob = np.concatenate([rk.get_spiked() for rk in ranks])
        for rk in ranks:
            rk.deliver_remote(glob)
    vm = np.concatenate([np.concatenate([s.vm for s in rk.solvers]) for rk in ranks])
    sp = np.concatenate([rk.net.spikes for rk in ranks])
    np.testing.assert_array_equal(sp, ref_sp)
    np.testing.assert_array_equal(vm, ref_vm)


def _gloo_worker(rank, world, port, out):
    sys.path.insert(0, os.path.join(REPO, "genesis-2.4_gb300"))
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from oracle_rank import OracleRank
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    import pyoracle
    dist.init_process_group("gloo", rank=rank, world_size=world)
    hs, esyn, child = _network(50, 0.12, seed=8)
    n = len(hs)
    lo, hi = shard.shard_range(n, rank, world)
    loc, rem = shard.partition_network(esyn, lo, hi, target_child=child)
    rk = OracleRank(pyoracle, hs[lo:hi], loc, rem)
    shard.run_partitioned(rk, 700, n, dist)
    vm = np.zeros(n * hs[0].ncompts)
    sp = np.zeros(n)
    vm[lo * hs[0].ncompts:hi * hs[0].ncompts] = np.concatenate([s.vm for s in rk.solvers])
    sp[lo:hi] = rk.net.spikes
    t = torch.from_numpy(np.concatenate([vm, sp]))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(out, t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_partitioned_oracle_two_gloo_ranks(oracle, tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "net.npy")
    port = 29700 + os.getpid() % 1000
    mp.start_processes(_gloo_worker, args=(2, port, out), nprocs=2, start_method="spawn")
    got = np.load(out)
    hs, esyn, child = _network(50, 0.12, seed=8)
    ref_vm, ref_sp = _oracle_whole(oracle, hs, esyn, child, 700)
    assert ref_sp.sum() > len(hs)
    np.testing.assert_array_equal(got[len(ref_vm):], ref_sp)
    np.testing.assert_array_equal(got[:len(ref_vm)], ref_vm)


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [False, True])
def test_partitioned_engines_match_oracle(oracle, gpu_engine, use_graph):
    hs, esyn, child = _network(90, 0.08, seed=12)
    n, nsteps, world = len(hs), 1200, 2
    ref_vm, ref_sp = _oracle_whole(oracle, hs, esyn, child, nsteps)
    assert ref_sp.sum() > n
    engs = []
    for r in range(world):
        lo, hi = shard.shard_range(n, r, world)
        loc, rem = shard.partition_network(esyn, lo, hi)
        engs.append(gpu_engine.Engine(hs[lo:hi], synapses=loc, remote=rem, use_graph=use_graph))
    for _ in range(nsteps):
        for e in engs:
            e.run(1)
        glob = np.concatenate([e.get_spiked() for e in engs])
        for e in engs:
            e.deliver_remote(glob)
    np.testing.assert_array_equal(np.concatenate([e.spike_counts() for e in engs]), ref_sp)
    np.testing.assert_array_equal(np.concatenate([e.vm() for e in engs]), ref_vm)
    for e in engs:
        e.close()


@pytest.mark.gpu
def test_partitioned_engines_weights_per_synapse(oracle, gpu_engine):
    """Weights per synapse across ranks: each rank sums the events due in a
    step in the global order (its first solver's global index places its own
    sources among the remote ones), so two engines equal the single-process
    oracle bit for bit."""
    hs, esyn, child = _network(90, 0.1, seed=14)
    rng = np.random.default_rng(15)
    ws = dict(esyn)
    ws["weight"] = rng.uniform(0.2, 2.0, size=len(esyn["weight"])).astype(np.float32).astype(np.float64)
    ws["delay_steps"] = rng.integers(1, 5, size=len(esyn["weight"])).astype(np.int32)
    n, nsteps, world = len(hs), 1200, 2
    ref_vm, ref_sp = _oracle_whole(oracle, hs, ws, child, nsteps)
    assert ref_sp.sum() > n
    engs = []
    for r in range(world):
        lo, hi = shard.shard_range(n, r, world)
        loc, rem = shard.partition_network(ws, lo, hi)
        engs.append(gpu_engine.Engine(hs[lo:hi], synapses=loc, remote=rem))
    for _ in range(nsteps):
        for e in engs:
            e.run(1)
        glob = np.concatenate([e.get_spiked() for e in engs])
        for e in engs:
            e.deliver_remote(glob)
    np.testing.assert_array_equal(np.concatenate([e.spike_counts() for e in engs]), ref_sp)
    np.testing.assert_array_equal(np.concatenate([e.vm() for e in engs]), ref_vm)
    for e in engs:
        e.close()


@pytest.mark.gpu
def test_partitioned_zero_delay_across_ranks_is_refused(gpu_engine):
    """A spike exchanged between steps cannot act in the step it happened."""
    hs, esyn, _ = _network(40, 0.2, seed=16)
    ws = dict(esyn)
    ws["delay_steps"] = np.zeros(len(esyn["weight"]), dtype=np.int32)
    loc, rem = shard.partition_network(ws, 20, 40)   # remote sources precede the rank's cells
    assert (rem["delay_steps"] == 0).any()
    with pytest.raises(gpu_engine.EngineError):
        gpu_engine.Engine(hs[20:40], synapses=loc, remote=rem)
