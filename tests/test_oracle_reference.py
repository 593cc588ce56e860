"""The CPU oracle against the reference's own step code and golden values.

* the reference's known answer: hh1952_ap_verify.g, 8 neurons, 10+200 steps,
  chanmode 4, CPU FP64 -> RESULT_VM= -0.02143485882
  (cluster_bringup/accel_regression_golden.txt:4), reproduced by the SETUP
  restatement plus the oracle, and checked against the committed fixture;
* where the reference sources are present (this build container), the
  oracle is checked bit for bit against do_chip_hh4_update /
  do_h4_conc_chip_update / do_euler_hsolve / do_crank_hsolve compiled from
  them (oracle/_ref), on single solvers and on a spiking network.
"""
import os

import numpy as np
import pytest

from gbhsolve import configs, model

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_ap_verify_golden(oracle):
    h = model.build(configs.ap_verify(8))
    s = oracle.Solver(h)
    s.run(210)
    assert "%0.10g" % s.vm[h.ncompts - 1] == configs.AP_VERIFY_GOLDEN


def test_golden_fixtures(oracle):
    """Committed fixtures: model arrays and the reference's own trajectory."""
    d = np.load(os.path.join(GOLDEN, "ref_trajectories.npz"), allow_pickle=False)
    names = [str(x) for x in d["names"]]
    for name in names:
        h = _from_npz(d, name)
        s = oracle.Solver(h)
        s.run(int(d[name + "/nsteps"]))
        np.testing.assert_array_equal(s.vm, d[name + "/vm_ref"])
        np.testing.assert_array_equal(s.chip, d[name + "/chip_ref"])


def _from_npz(d, name):
    from types import SimpleNamespace
    g = lambda k: d[name + "/" + k]
    sc = g("scalars")
    return SimpleNamespace(
        ncompts=int(sc[0]), ops=g("ops"), chip=g("chip"), funcs=g("funcs"), ravals=g("ravals"), vm=g("vm"),
        givals=g("givals"), ncols=int(sc[1]), xdivs=int(sc[2]), xmin=float(sc[3]), invdx=float(sc[4]),
        tablist=g("tablist"), xvals=g("xvals"), ydivs=int(sc[5]), ymin=float(sc[6]), invdy=float(sc[7]),
        yvals=g("yvals"), stablist=g("stablist"), conc=g("conc"), concops=g("concops"),
        concchip=g("concchip"), childops=g("childops"), childchips=g("childchips"), dt=float(sc[8]),
        crank=int(sc[9]), chanmode=int(sc[10]), calcmode=int(sc[11]), method=11 if int(sc[9]) else 10)


needs_ref = pytest.mark.skipif(not os.path.exists("/root/reference/genesis/src/hines/hines_chip.c"),
                               reason="reference sources not present")


@needs_ref
@pytest.mark.parametrize("method", [model.BEULER, model.CRANK])
def test_oracle_matches_reference_step_code(oracle, method):
    oracle.ensure_built(with_reference=True)
    for m in (configs.cables(12, gk_dend=36.0, method=method)[0],
              configs.random_trees(1, size_range=(40, 40), seed=3, method=method)[0]):
        h = model.build(m)
        a, b = oracle.Solver(h), oracle.Solver(h)
        a.run(300, "oracle")
        b.run(300, "reference")
        np.testing.assert_array_equal(a.vm, b.vm)
        np.testing.assert_array_equal(a.chip, b.chip)
        np.testing.assert_array_equal(a.conc, b.conc)


@needs_ref
def test_oracle_network_matches_reference_step_code(oracle):
    oracle.ensure_built(with_reference=True)
    ms, syn = configs.hh_network(40, p_conn=0.2, seed=2)
    rng = np.random.default_rng(0)
    for m in ms:
        m.compartments[0].inject = float(rng.uniform(0, 0.3e-9))
    hs = [model.build(m) for m in ms]
    esyn, child = configs.network_synapses(hs, syn)
    runs = []
    for impl in ("oracle", "reference"):
        sv = [oracle.Solver(h, i) for i, h in enumerate(hs)]
        net = oracle.Network(sv, esyn["src_start"], esyn["target_solver"], child, esyn["target_op"],
                             esyn["weight"], esyn["delay_steps"], impl=impl)
        net.run(1500)
        runs.append((np.concatenate([s.vm for s in sv]), net.spikes.copy()))
    assert runs[0][1].sum() > 0
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
