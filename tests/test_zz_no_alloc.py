"""gbh_run_noalloc: the step entry point that allocates no device memory.

It is for hosts that may not allocate device memory while stepping: the
GPU's memory was reserved at start-up by a pool another runtime owns, or
the step loop cannot afford cudaMalloc/cudaFree, which may synchronise the
whole device. Its Ca-flux scratch is a fixed array inside the library, so
this test uses a model with Ca pools, where that scratch is really used, and
checks two consecutive calls against gbh_run on an identical engine. The
FP64 step is exact, so the comparison is bit for bit, the same tolerance the
other FP64 engine tests use. This file is collected last on purpose.
"""
import numpy as np
import pytest
import torch

from gbhsolve import configs, model

pytestmark = pytest.mark.gpu


def test_run_noalloc_matches_run_twice(gpu_engine):
    hs = [model.build(m) for m in configs.random_trees(40, size_range=(8, 48), seed=11)]
    ref = gpu_engine.Engine(hs, steps_per_launch=25)
    new = gpu_engine.Engine(hs, steps_per_launch=25)
    for _ in range(2):
        ref.run(120)
        new.run_noalloc(120)          # queued on the default stream
        a = ref.get_state()           # get_state synchronises the device copy
        torch.cuda.synchronize()
        b = new.get_state()
        for i in range(len(hs)):
            np.testing.assert_array_equal(b["vm"][i], a["vm"][i])
            np.testing.assert_array_equal(b["conc"][i], a["conc"][i])
            np.testing.assert_array_equal(b["chip"][i], a["chip"][i])
    ref.close()
    new.close()
