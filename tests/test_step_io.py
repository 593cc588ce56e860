"""gbh_step_io (pipelined per-step inputs and outputs) against the plain
per-step calls: same outputs step by step (the pipelined ones complete two
calls later) and the same final state, with inputs that change every step."""
import numpy as np
import pytest

from gbhsolve import configs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pinned", [False, True])
def test_step_io_matches_plain_calls(gpu_engine, pinned):
    import torch
    hs, injects = configs.cables_replicated(300, gk_dend=36.0, seed=4)
    n = len(hs)
    slot = configs.inject_slot(hs[0])
    soma = hs[0].ncompts - 1
    engs = []
    for _ in range(2):
        e = gpu_engine.Engine(hs, precision=gpu_engine.PREC_MIXED, steps_per_launch=1)
        e.register_inputs(np.arange(n, dtype=np.int32), np.full(n, slot, dtype=np.int64))
        e.register_outputs(np.arange(n, dtype=np.int32), np.full(n, soma, dtype=np.int32))
        engs.append(e)
    plain, piped = engs
    rng = np.random.default_rng(0)
    nsteps = 400
    inputs = rng.uniform(0.0, 0.6e-9, size=(nsteps, n))
    ref = np.empty((nsteps, n))
    buf = np.empty(n)
    for k in range(nsteps):
        plain.set_inputs_async(np.ascontiguousarray(inputs[k]), 0)
        plain.run(1)
        plain.get_outputs_async(buf, 0)
        plain.vm()                                  # synchronises the engine stream
        ref[k] = buf
    if pinned:
        ins = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
        outs = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    else:
        ins = [np.empty(n) for _ in range(3)]
        outs = [np.empty(n) for _ in range(3)]
    got = np.empty((nsteps, n))
    for k in range(nsteps):
        ins[k % 3][:] = inputs[k]                     # reused three calls later
        piped.step_io(ins[k % 3], outs[k % 3], 1)
        if k >= 2:
            got[k - 2] = outs[(k - 2) % 3]            # complete once call k has returned
    piped.io_sync()
    for k in (nsteps - 2, nsteps - 1):
        got[k] = outs[k % 3]
    np.testing.assert_array_equal(got, ref)
    np.testing.assert_array_equal(piped.vm(), plain.vm())
    for e in engs:
        e.close()


@pytest.mark.parametrize("block,pinned", [(0, True), (7, False), (1, True), (64, True)])
def test_run_io_matches_plain_calls(gpu_engine, block, pinned):
    """gbh_run_io streams a whole run's per-step inputs and outputs in blocks
    (ragged last block for block 7 and 64 over 150 steps): outputs step by
    step and the final state equal the plain per-step calls."""
    import torch
    hs, _ = configs.cables_replicated(200, gk_dend=36.0, seed=6)
    n = len(hs)
    slot = configs.inject_slot(hs[0])
    soma = hs[0].ncompts - 1
    engs = []
    for _ in range(2):
        e = gpu_engine.Engine(hs, precision=gpu_engine.PREC_MIXED, steps_per_launch=1)
        e.register_inputs(np.arange(n, dtype=np.int32), np.full(n, slot, dtype=np.int64))
        e.register_outputs(np.arange(n, dtype=np.int32), np.full(n, soma, dtype=np.int32))
        engs.append(e)
    plain, streamed = engs
    nsteps = 150
    inputs = np.random.default_rng(1).uniform(0.0, 0.6e-9, size=(nsteps, n))
    ref = np.empty((nsteps, n))
    buf = np.empty(n)
    for k in range(nsteps):
        plain.set_inputs_async(np.ascontiguousarray(inputs[k]), 0)
        plain.run(1)
        plain.get_outputs_async(buf, 0)
        plain.vm()
        ref[k] = buf
    if pinned:
        hin = torch.empty((nsteps, n), dtype=torch.float64, pin_memory=True).numpy()
        hout = torch.empty((nsteps, n), dtype=torch.float64, pin_memory=True).numpy()
    else:
        hin, hout = np.empty((nsteps, n)), np.empty((nsteps, n))
    hin[:] = inputs
    streamed.run_io(hin, hout, nsteps, block=block)
    np.testing.assert_array_equal(hout, ref)
    np.testing.assert_array_equal(streamed.vm(), plain.vm())
    # outputs only, then inputs only: the state keeps matching
    streamed.run_io(None, hout, 5, block=block)
    for k in range(5):
        plain.run(1)
        plain.get_outputs_async(buf, 0)
        plain.vm()
        np.testing.assert_array_equal(hout[k], buf)
    streamed.run_io(hin, None, 3, block=block)
    for k in range(3):
        plain.set_inputs_async(np.ascontiguousarray(inputs[k]), 0)
        plain.run(1)
    np.testing.assert_array_equal(streamed.vm(), plain.vm())
    for e in engs:
        e.close()
