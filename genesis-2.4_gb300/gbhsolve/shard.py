"""Neuron sharding across ranks (one process per GPU).

Neurons are independent block-diagonal systems, so a model shards by
contiguous neuron ranges with no exchange on the data path; only results
(step time, spike counts, losses) are reduced at the end.
"""
from __future__ import annotations


def shard_range(n_items: int, rank: int, world: int):
    """Contiguous [lo, hi) share of n_items for rank (sizes differ by <= 1)."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(n_items, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def reduce_max(value: float, dist=None) -> float:
    """Max over ranks (the job's time is its slowest rank's)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(values, dist=None):
    if dist is None:
        return values
    import torch
    t = torch.as_tensor(values, dtype=torch.float64).clone()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.numpy()


# --------------------------------------------------------------------------
# Partitioned spiking networks: cells split into contiguous ranges, one range
# per rank; spikes are all-gathered every step and delivered on each rank.
# --------------------------------------------------------------------------
def partition_network(syn, lo, hi, spike_op=None, target_child=None):
    """Synapse tables of the rank owning solvers [lo, hi) of a network.

    ``syn``: the whole network's table (CSR over source solvers:
    src_start, target_solver, target_op, weight, delay_steps; see
    configs.network_synapses). Returns (local, remote):
      local   synapses with both ends on this rank, CSR over local sources,
              solver indices counted from lo (the engine applies the in-step
              ordering rule itself, which keeps the global order within a
              contiguous range);
      remote  synapses from cells of other ranks to this rank's cells, CSR
              over all n sources (global index; a local source's range is
              empty), first_solver = lo, target solvers counted from lo,
              effective delays: the
              delay plus 1 when the target's global index precedes the
              source's (the reference steps solvers in order, so such a
              target sees the spike one step later).
    ``target_child`` (optional, per synapse): carried into both tables as
    'target_child' for the oracle's network layer."""
    import numpy as np
    start = np.asarray(syn["src_start"], dtype=np.int64)
    n = len(start) - 1
    ts = np.asarray(syn["target_solver"])
    keys = ["target_solver", "target_op", "weight", "delay_steps"]
    loc = {k: [] for k in keys + ["target_child"]}
    rem = {k: [] for k in keys + ["target_child"]}
    loc_start, rem_start = [0], [0]
    for s in range(n):
        for k in range(start[s], start[s + 1]):
            t = int(ts[k])
            if not (lo <= t < hi):
                continue
            dst = loc if lo <= s < hi else rem
            dst["target_solver"].append(t - lo)
            dst["target_op"].append(int(syn["target_op"][k]))
            dst["weight"].append(float(syn["weight"][k]))
            d = int(syn["delay_steps"][k])
            if dst is rem and t < s:
                d += 1
            dst["delay_steps"].append(d)
            dst["target_child"].append(int(target_child[k]) if target_child is not None else -1)
        if lo <= s < hi:
            loc_start.append(len(loc["weight"]))
        rem_start.append(len(rem["weight"]))
    local = {"src_start": np.asarray(loc_start, dtype=np.int64)}
    remote = {"src_start": np.asarray(rem_start, dtype=np.int64), "first_solver": int(lo)}
    for k, t in (("target_solver", np.int32), ("target_op", np.int32), ("weight", np.float64),
                 ("delay_steps", np.int32), ("target_child", np.int32)):
        local[k] = np.asarray(loc[k], dtype=t)
        remote[k] = np.asarray(rem[k], dtype=t)
    return local, remote


def gather_spikes(mine, n_global, dist=None):
    """All-gather the ranks' spike flags (bool per local cell, contiguous
    ranges as shard_range gives them) as packed bitmaps; returns the bool
    array over all n_global cells."""
    import numpy as np
    mine = np.asarray(mine, dtype=bool)
    if dist is None:
        return mine
    import torch
    world = dist.get_world_size()
    sizes = [shard_range(n_global, r, world) for r in range(world)]
    width = max(hi - lo for lo, hi in sizes)
    buf = np.zeros((width + 7) // 8, dtype=np.uint8)
    packed = np.packbits(mine, bitorder="little")
    buf[:len(packed)] = packed
    t = torch.from_numpy(buf)
    out = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(out, t)
    parts = [np.unpackbits(o.numpy(), bitorder="little")[:hi - lo] for o, (lo, hi) in zip(out, sizes)]
    return np.concatenate(parts).astype(bool)


def run_partitioned(rank_sim, nsteps, n_global, dist=None):
    """Steps a rank's simulator (an Engine, or any object with run /
    get_spiked / deliver_remote) with one spike exchange per step."""
    for _ in range(nsteps):
        rank_sim.run(1)
        rank_sim.deliver_remote(gather_spikes(rank_sim.get_spiked(), n_global, dist))
