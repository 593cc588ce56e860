"""GPU engine vs the CPU oracle on identical models (FP64: bit for bit)."""
import numpy as np
import pytest

from gbhsolve import configs, model

pytestmark = pytest.mark.gpu


def _oracle_run(oracle, h, nsteps):
    s = oracle.Solver(h)
    s.run(nsteps)
    return s


def test_ap_verify_golden_fp64(oracle, gpu_engine):
    h = model.build(configs.ap_verify(8))
    eng = gpu_engine.Engine([h])
    eng.run(10)
    eng.run(200)
    vm = eng.vm()
    assert "%0.10g" % vm[h.ncompts - 1] == configs.AP_VERIFY_GOLDEN
    ref = _oracle_run(oracle, h, 210)
    np.testing.assert_array_equal(vm, ref.vm)


@pytest.mark.parametrize("method", [model.BEULER, model.CRANK])
@pytest.mark.parametrize("gk_dend", [0.0, 36.0])
def test_cables_single_hsolve_bitwise(oracle, gpu_engine, method, gk_dend):
    h = model.build(configs.cables(40, method=method, gk_dend=gk_dend)[0])
    eng = gpu_engine.Engine([h], steps_per_launch=37)
    eng.run(200)
    st = eng.get_state()
    ref = _oracle_run(oracle, h, 200)
    np.testing.assert_array_equal(st["vm"][0], ref.vm)
    np.testing.assert_array_equal(st["chip"][0], ref.chip)


def test_cables_per_neuron_solvers_bitwise(oracle, gpu_engine):
    hs = [model.build(m) for m in configs.cables(70, gk_dend=36.0, per_neuron_solvers=True)]
    eng = gpu_engine.Engine(hs)
    eng.run(150)
    st = eng.get_state()
    for i in (0, 33, 69):
        ref = _oracle_run(oracle, hs[i], 150)
        np.testing.assert_array_equal(st["vm"][i], ref.vm)
        np.testing.assert_array_equal(st["chip"][i], ref.chip)


def test_random_trees_with_ca_bitwise(oracle, gpu_engine):
    hs = [model.build(m) for m in configs.random_trees(48, size_range=(8, 64), seed=7)]
    eng = gpu_engine.Engine(hs, steps_per_launch=50)
    eng.run(300)
    st = eng.get_state()
    for i in range(0, 48, 5):
        ref = _oracle_run(oracle, hs[i], 300)
        np.testing.assert_array_equal(st["vm"][i], ref.vm)
        np.testing.assert_array_equal(st["conc"][i], ref.conc[:len(hs[i].conc)])


@pytest.mark.parametrize("jit", [True, False, 2, 3])
def test_jit_and_interpreter_agree_bitwise(oracle, gpu_engine, jit):
    """Both execution paths -- programs specialised at setup and the
    interpreting kernel -- reproduce the oracle exactly."""
    hs = configs.cables_replicated(50, gk_dend=36.0, seed=9)[0]
    hs += [model.build(m) for m in configs.random_trees(20, size_range=(10, 30), seed=2)]
    eng = gpu_engine.Engine(hs, jit=jit, steps_per_launch=40)
    eng.run(120)
    st = eng.get_state()
    for i in (0, 17, 49, 50, 60, 69):
        ref = _oracle_run(oracle, hs[i], 120)
        np.testing.assert_array_equal(st["vm"][i], ref.vm)
        np.testing.assert_array_equal(st["chip"][i], ref.chip)


def test_engine_matches_reference_fixtures(gpu_engine):
    """GPU engine against trajectories produced by the reference's own step
    code (tests/golden/make_golden.py): Euler, Crank-Nicolson, calcmode 0,
    a branched tree with a Ca pool."""
    import os
    from test_oracle_reference import _from_npz
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_trajectories.npz"))
    for name in [str(x) for x in d["names"]]:
        h = _from_npz(d, name)
        for jit in (True, False):
            eng = gpu_engine.Engine([h], jit=jit)
            eng.run(int(d[name + "/nsteps"]))
            st = eng.get_state()
            np.testing.assert_array_equal(st["vm"][0], d[name + "/vm_ref"], err_msg=name)
            np.testing.assert_array_equal(st["chip"][0], d[name + "/chip_ref"], err_msg=name)
            eng.close()
