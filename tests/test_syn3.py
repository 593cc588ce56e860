"""SYN3_OP (randomly triggered synchan, channelC3, hines_chip.c:511-531) on
the GPU: each neuron and step draws from a counter-based hash of (neuron,
step, synchan) instead of the reference's one sequential stream (G_RNG), so
parity is statistical: firing counts over many steps follow Binomial(N, p),
the criterion the reference's own generator meets
(tests/test_oracle_reference.py::test_syn3_oracle_firing_statistics)."""
import numpy as np
import pytest

import opprograms as P
from test_oracle_reference import check_binomial

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_syn3_firing_statistics(gpu_engine, precision):
    n, nsteps, p = 320, 2000, 0.1
    h = P.syn3_solver(p, [1.0, 0.0, 0.0, 1.0])
    eng = gpu_engine.Engine([h] * n, precision=precision)
    eng.run(nsteps)
    chips = eng.get_state()["chip"]
    counts = np.array([c[5] for c in chips])
    check_binomial(counts, nsteps, p)
    eng.close()
