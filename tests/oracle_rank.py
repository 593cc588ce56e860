"""One rank of a partitioned network on the CPU oracle, for the tests of the
partition and spike-exchange logic (gbhsolve/shard.py) without a GPU.

TEST INFRASTRUCTURE ONLY: it drives the oracle (orc_net over the rank's
solvers plus events delivered from the other ranks' spikes), the
reference's semantics, through the same run / get_spiked / deliver_remote
calls an Engine answers.
"""
import numpy as np


class OracleRank:
    """One rank of a partitioned network on the CPU oracle (orc_net over the
    rank's solvers plus events delivered from the other ranks' spikes): the
    reference's semantics for checking the exchange logic without a GPU."""

    def __init__(self, oracle, hs_local, local, remote):
        self.solvers = [oracle.Solver(h, i) for i, h in enumerate(hs_local)]
        self.net = oracle.Network(self.solvers, local["src_start"], local["target_solver"], local["target_child"],
                                  local["target_op"], local["weight"], local["delay_steps"])
        self.remote = remote
        self.last = np.zeros(len(hs_local), dtype=np.int64)

    def run(self, nsteps):
        self.net.run(nsteps)

    def get_spiked(self):
        now = self.net.spikes.copy()
        out = now > self.last
        self.last = now
        return out

    def deliver_remote(self, spiked):
        r = self.remote
        src = np.nonzero(spiked)[0]
        idx = np.concatenate([np.arange(r["src_start"][s], r["src_start"][s + 1]) for s in src]) \
            if len(src) else np.zeros(0, dtype=np.int64)
        if len(idx):
            step = self.net.step - 1
            self.net.deliver(r["target_solver"][idx], r["target_child"][idx], r["target_op"][idx],
                             r["weight"][idx], step + r["delay_steps"][idx].astype(np.int64))
