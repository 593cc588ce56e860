"""Mixed-precision form (double-float gates on FP32, FP64 elimination/Vm/Ca)
against the FP64 CPU oracle. Tolerance: max|dVm| <= 1e-6 V over the run."""
import numpy as np
import pytest

from gbhsolve import configs, model

pytestmark = pytest.mark.gpu

TOL_V = 1e-6


def _max_dev(oracle, gpu_engine, hs, nsteps, chunk=500, **kw):
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_MIXED, **kw)
    orc = [oracle.Solver(h) for h in hs]
    worst = 0.0
    done = 0
    while done < nsteps:
        k = min(chunk, nsteps - done)
        eng.run(k)
        for s in orc:
            s.run(k)
        vm = eng.vm()
        worst = max(worst, float(np.max(np.abs(vm - np.concatenate([s.vm for s in orc])))))
        done += k
    eng.close()
    return worst


@pytest.mark.parametrize("jit", [True, False, 2, 3])
def test_mixed_cables_10k_steps(oracle, gpu_engine, jit):
    hs, _ = configs.cables_replicated(32, gk_dend=36.0, seed=3)
    dev = _max_dev(oracle, gpu_engine, hs, 10000, jit=jit)
    assert dev <= TOL_V, dev


@pytest.mark.parametrize("method", [model.BEULER, model.CRANK])
def test_mixed_single_hsolve_many_neurons(oracle, gpu_engine, method):
    h = model.build(configs.cables(20, method=method, gk_dend=36.0)[0])
    assert _max_dev(oracle, gpu_engine, [h], 3000) <= TOL_V


def test_mixed_random_trees_with_ca(oracle, gpu_engine):
    hs = [model.build(m) for m in configs.random_trees(40, size_range=(8, 64), seed=5)]
    assert _max_dev(oracle, gpu_engine, hs, 3000) <= TOL_V
