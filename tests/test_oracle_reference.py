"""The CPU oracle against the reference's own step code and golden values.

* the reference's known answer: hh1952_ap_verify.g, 8 neurons, 10+200 steps,
  chanmode 4, CPU FP64 -> RESULT_VM= -0.02143485882
  (cluster_bringup/accel_regression_golden.txt:4), reproduced by the SETUP
  restatement plus the oracle, and checked against the committed fixture;
* where the reference sources are present, the
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


import pyoracle  # noqa: E402

needs_ref = pytest.mark.skipif(not pyoracle.reference_sources_present(), reason="reference sources not present")


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


def test_opcode_programs_equal_reference_fixture(oracle):
    """Every opcode program of tests/opprograms.py in all three step modes:
    the oracle against the reference's own step code (committed fixture)."""
    import opprograms as P
    d = np.load(os.path.join(GOLDEN, "ref_opcodes.npz"), allow_pickle=False)
    tags = [str(t) for t in d["tags"]]
    assert len(tags) == len(P.PROGRAMS) * len(P.MODES)
    for name in sorted(P.PROGRAMS):
        for mode in P.MODES:
            h, libm = P.build(name, *mode)
            tag = P.mode_tag(name, *mode)
            assert str(d[tag + "/digest"]) == P.input_digest(h), tag
            hf = P.from_fixture(d, tag)
            assert P.input_digest(hf) == P.input_digest(h), tag
            s = oracle.Solver(hf)
            s.run(int(d["nsteps"]))
            for k in ("vm", "chip", "givals"):
                if libm:    # exp/log: libm of the machine running the test
                    np.testing.assert_allclose(getattr(s, k), d[tag + "/" + k], rtol=1e-12, atol=1e-18,
                                               err_msg=tag)
                else:
                    np.testing.assert_array_equal(getattr(s, k), d[tag + "/" + k], err_msg=tag)
            np.testing.assert_array_equal(s.ops, d[tag + "/ops"], err_msg=tag)
            if len(h.conc):
                np.testing.assert_allclose(s.conc[:len(h.conc)], d[tag + "/conc"], rtol=1e-12 if libm else 0,
                                           atol=0, err_msg=tag)


@needs_ref
def test_opcode_programs_oracle_equals_live_reference(oracle):
    """The same programs run live through the compiled reference here."""
    import opprograms as P
    oracle.ensure_built(with_reference=True)
    for name in sorted(P.PROGRAMS):
        for mode in P.MODES:
            h, _ = P.build(name, *mode)
            a, b = oracle.Solver(h), oracle.Solver(h)
            a.run(P.NSTEPS, "oracle")
            b.run(P.NSTEPS, "reference")
            for k in ("vm", "chip", "conc", "givals", "ops"):
                np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=P.mode_tag(name, *mode))


def test_domain_without_concentrations_is_a_setup_error():
    """DOMAIN_OP needs the concentration axis, which a solver has only when it
    holds concentrations (hines_chip.c:131-140); the reference would read
    through a NULL yvals, the engine refuses the model at setup."""
    import ophelpers as A
    import opprograms as P
    from gbhsolve import engine
    c = P._c()
    c.op(A.NEWVOLT).op(A.CHAN_EK, chips=[0.1, 1e-8]).op(A.IPOL1V, 0, 2, chips=[0.3]).op(A.ADD_CURR, giv=3)
    c.op(A.DOMAIN, chips=[1e7]).op(A.CHAN_EK, chips=[-0.08, 2e-8]).op(A.IPOL1C, 4, 1, chips=[0.2])
    c.op(A.ADD_CURR, giv=3)
    h = A.solver([c], A.tables(12, 40, seed=7, ydivs=40), dt=P.DT)
    with pytest.raises(engine.EngineError) as ei:
        engine.validate([h])
    assert ei.value.opcode == A.DOMAIN


@needs_ref
def test_oracle_network_weights_zero_delay_matches_reference_step_code(oracle):
    """Per-synapse weights and zero-step delays through the reference's own
    step code (do_chip_hh4_update calling h_dosynchan) under the oracle's
    event layer, against the oracle's own step."""
    oracle.ensure_built(with_reference=True)
    ms, syn = configs.hh_network(40, p_conn=0.2, seed=3)
    rng = np.random.default_rng(1)
    for m in ms:
        m.compartments[0].inject = float(rng.uniform(0, 0.3e-9))
    hs = [model.build(m) for m in ms]
    esyn, child = configs.network_synapses(hs, syn)
    w = rng.uniform(0.2, 2.0, size=len(esyn["weight"])).astype(np.float32).astype(np.float64)
    d = rng.integers(0, 4, size=len(w)).astype(np.int32)
    runs = []
    for impl in ("oracle", "reference"):
        sv = [oracle.Solver(h, i) for i, h in enumerate(hs)]
        net = oracle.Network(sv, esyn["src_start"], esyn["target_solver"], child, esyn["target_op"], w, d,
                             impl=impl)
        net.run(1500)
        runs.append((np.concatenate([s.vm for s in sv]), net.spikes.copy()))
    assert runs[0][1].sum() > 0
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])


@needs_ref
def test_syn3_draws_equal_reference_generator(oracle):
    """SYN3_OP (channelC3) draws urandom() = G_RNG() each step; the oracle's
    restatement of GENESIS's default generator (Numerical Recipes ran1) gives
    the reference's own sim/sim_random.c stream: equal trajectories from the
    same seed."""
    import opprograms as P
    oracle.ensure_built(with_reference=True)
    h = P.syn3_solver(0.1, [0.99, 9.5e-5, 0.98, 9.9e-5 / P.DT], n_compts=3)
    runs = []
    for impl in ("oracle", "reference"):
        oracle.seed_rng(7, impl)
        s = oracle.Solver(h)
        s.run(3000, impl)
        runs.append((s.vm.copy(), s.chip.copy()))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
    assert runs[0][1][5] != 0.0


def test_syn3_oracle_firing_statistics(oracle):
    """The criterion the engine's SYN3 draws are held to, applied to the
    reference's generator (restated): X counts firings exactly when
    xconst2 = 1 and the increment is 1; counts are Binomial(N, p)."""
    import opprograms as P
    n, nsteps, p = 96, 2000, 0.1
    h = P.syn3_solver(p, [1.0, 0.0, 0.0, 1.0], n_compts=n)
    oracle.seed_rng(3)
    s = oracle.Solver(h)
    s.run(nsteps)
    counts = s.chip[5::9][:n]
    check_binomial(counts, nsteps, p)


def check_binomial(counts, nsteps, p):
    counts = np.asarray(counts)
    assert np.all(counts == np.round(counts))
    mean, var = nsteps * p, nsteps * p * (1 - p)
    assert abs(counts.mean() - mean) < 5 * np.sqrt(var / len(counts)), counts.mean()
    assert 0.6 * var < counts.var() < 1.5 * var, counts.var()
    assert len(np.unique(counts)) > 10          # neurons draw independent streams
