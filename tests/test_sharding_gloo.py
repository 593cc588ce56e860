"""Weak-scaling path on CPU ranks: two gloo processes shard a cable
population by neuron, each steps its shard with the oracle, and the reduced
result equals the single-process run (no data-path exchange is needed)."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_range_partition():
    from gbhsolve.shard import shard_range
    for n in (1, 7, 100, 101):
        for w in (1, 2, 3, 8):
            got = [shard_range(n, r, w) for r in range(w)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))


def _worker(rank, world, port, out):
    sys.path.insert(0, os.path.join(REPO, "genesis-2.4_gb300"))
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import pyoracle
    from gbhsolve import configs
    from gbhsolve.shard import reduce_max, reduce_sum, shard_range
    dist.init_process_group("gloo", rank=rank, world_size=world)
    hs, _ = configs.cables_replicated(10, gk_dend=36.0, seed=1)
    lo, hi = shard_range(len(hs), rank, world)
    vm = np.zeros(len(hs) * 16)
    for i in range(lo, hi):
        s = pyoracle.Solver(hs[i])
        s.run(150)
        vm[i * 16:(i + 1) * 16] = s.vm
    tot = reduce_sum(vm, dist)
    t = reduce_max(float(rank + 1), dist)
    if rank == 0:
        np.save(out, np.concatenate([tot, [t]]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_shards_match_single_process(tmp_path):
    import torch.multiprocessing as mp
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    from gbhsolve import configs
    pyoracle.ensure_built(with_reference=False)
    out = str(tmp_path / "vm.npy")
    port = 29500 + os.getpid() % 1000
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, start_method="spawn")
    got = np.load(out)
    hs, _ = configs.cables_replicated(10, gk_dend=36.0, seed=1)
    ref = []
    for h in hs:
        s = pyoracle.Solver(h)
        s.run(150)
        ref.append(s.vm)
    np.testing.assert_array_equal(got[:-1], np.concatenate(ref))
    assert got[-1] == 2.0
