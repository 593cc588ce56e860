"""Concentration diffusion systems (difshells with fixed and diffusible
buffers, pumps, concpools): the concops program of do_h4_conc_chip_update
(hines_conc_chip.c:59-221) and the shell/buffer solve of do_h_conc_solve
(hines_conc.c:39-396), on hand-assembled hsolves.

CPU: the oracle restatement equals the reference's own compiled code
(oracle/_ref) bit for bit. GPU: the engine equals the oracle bit for bit in
FP64 and within 1e-9 V / 1e-12 mM in the mixed form."""
import numpy as np
import pytest

import ophelpers as A

DT = 2e-5


def _cell(vm0=-0.055, inj=2e-10):
    c = A.Compt(emrm=-0.065 / 1e9, inject=inj, tbyc=DT / 1e-11, diag=1.0 + DT / 1e-11 / 1e9, rm=1e9, vm0=vm0)
    # K-like channel, a Ca channel whose current feeds conc `ca`, a Ca-gated channel
    c.op(A.NEWVOLT).op(A.CHAN_EK, chips=[-0.08, 4e-9]).op(A.IPOL1V, 0, 4, chips=[0.3]).op(A.ADD_CURR, giv=3)
    return c


def _ca_ops(c, ca):
    c.op(A.CONC_VAL, ca).op(A.CHAN_EK, chips=[0.12, 8e-10]).op(A.IPOL1V, 2, 2, chips=[0.1]).op(A.ADD_CURR, giv=3)
    c.op(A.FLUX).op(A.NEWCONC1).op(A.CHAN_EK, chips=[-0.08, 3e-9]).op(A.IPOL1C, 4, 1, chips=[0.2])
    c.op(A.ADD_CURR, giv=3)
    return c


def prog_shells(crank):
    """Five shells, no buffers: flux leak, MM, tau, Hill and voltage-tau pumps."""
    rng = np.random.default_rng(1)
    cov0, _, conc = A.diffusion_system(rng, 5, dt=DT, crank=crank)
    c = _ca_ops(_cell(), 0)
    ops = [A.FCONC, 0, A.FLUXCONC, A.MMPUMP, A.CTAUPUMP, A.CONC, 2, A.HILLPUMP, 2, A.CONC, 3, A.TAUPUMP, 0,
           A.CONC, 4, A.HILLPUMP, 1, A.LCONC]
    chips = [1e-9, 5e5, 1e-6, 1e-3, 5e-8, 1e-3, 1e-3, 2e-6, 0.02, 0.01, -0.05, 50.0, 5e-5, 2e-4, 3e-7]
    diff = dict(dconc=[0], nshells=[5], nshrows=[1], nshfix=[0], fbufval=[0], covals0=cov0, bufvals=[])
    return [c], dict(conc=conc, concops=ops, concchip=chips, diff=diff)


def prog_buffers():
    """Four shells with a fixed and a diffusible buffer, an electrogenic pump
    on the first shell, and a buffered concpool fed by a Hill pump from the
    third shell (Crank-Nicolson: GENESIS solves buffers with it only)."""
    rng = np.random.default_rng(2)
    cov0, bufv, conc = A.diffusion_system(rng, 4, nfix=1, ndif=1, dt=DT, crank=True)
    c = _ca_ops(_cell(), 2)
    c.op(A.CONC_VAL, 2).op(A.ELMMPUMP, chips=[2e-4, 3e-13, 4e-4], giv=1)
    conc = list(conc) + [2e-4, 0.05]            # pool, its buffer
    ops = [A.FCONC, 2, A.FLUXCONC, A.CONC, 5, A.MMPUMP, A.CONC, 11, A.CTAUPUMP,
           A.CONC, 12, A.PHILLPUMP, 3, 8, A.BUFFER, 13, A.POOL, A.LCONC]
    chips = [2e-9, 4e5, 1e-6, 1e-3, 4e-8, 8e-4, 1e-3, 2e-6, 1e-6, 0.5 * DT * 100.0, DT * 100.0 * 0.1, DT * 2e5]
    diff = dict(dconc=[0], nshells=[4], nshrows=[3], nshfix=[1], fbufval=[0], covals0=cov0, bufvals=bufv)
    return [c], dict(conc=conc, concops=ops, concchip=chips, diff=diff)


def prog_two_systems():
    """Two compartments, each with its own system (shells only, then
    buffered), covals0 consumed across both."""
    rng = np.random.default_rng(3)
    cov_a, _, conc_a = A.diffusion_system(rng, 3, dt=DT, crank=True)
    cov_b, bufv, conc_b = A.diffusion_system(rng, 3, nfix=0, ndif=2, dt=DT, crank=True)
    ca_b = len(conc_a) + 2                       # first shell Ca of system b
    c0 = _ca_ops(_cell(), 0)
    c1 = _ca_ops(_cell(-0.06, 1e-10), ca_b)
    ops = [A.FCONC, 0, A.FLUXCONC, A.CONC, ca_b, A.FLUXCONC, A.CTAUPUMP, A.LCONC]
    chips = [0.0, 6e5, 1e-9, 3e5, 5e-8, 1e-3]
    diff = dict(dconc=[0, len(conc_a)], nshells=[3, 3], nshrows=[1, 3], nshfix=[0, 0], fbufval=[0, 0],
                covals0=np.concatenate([cov_a, cov_b]), bufvals=bufv)
    return [c0, c1], dict(conc=list(conc_a) + list(conc_b), concops=ops, concchip=chips, diff=diff,
                          parents=[1, -1])


PROGRAMS = {"shells_euler": lambda: prog_shells(False), "shells_crank": lambda: prog_shells(True),
            "buffers": prog_buffers, "two_systems": prog_two_systems}
CRANK = {"shells_euler": False, "shells_crank": True, "buffers": True, "two_systems": True}


def build(name):
    compts, kw = PROGRAMS[name]()
    tabs = A.tables(12, 40, seed=21, ydivs=40, ymax=2e-3)
    return A.solver(compts, tabs, dt=DT, crank=CRANK[name], **kw)


@pytest.mark.parametrize("name", sorted(PROGRAMS))
def test_oracle_equals_reference(oracle, name):
    """The C restatement against the reference's own do_h4_conc_chip_update
    and do_h_conc_solve (compiled from its sources), bit for bit."""
    if not oracle.reference_sources_present():
        pytest.skip("reference sources not present")
    h = build(name)
    a, b = oracle.Solver(h), oracle.Solver(h)
    for _ in range(20):
        a.run(50)
        b.run(50, impl="ref")
        np.testing.assert_array_equal(a.conc, b.conc)
        np.testing.assert_array_equal(a.vm, b.vm)
        np.testing.assert_array_equal(a.chip, b.chip)
    # the run moved the shells apart (the system is not at rest)
    assert np.ptp(a.conc[:len(h.conc)]) > 0


LIBM = {"shells_euler", "shells_crank"}   # TAUPUMP_OP's exp: CUDA against libm, to the last bits


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [True, False])
@pytest.mark.parametrize("name", sorted(PROGRAMS))
def test_engine_fp64_equals_oracle(oracle, gpu_engine, name, jit):
    h = build(name)
    eng = gpu_engine.Engine([h], jit=jit)
    ref = oracle.Solver(h)
    for _ in range(4):
        eng.run(250)
        ref.run(250)
        st = eng.get_state()
        if name in LIBM:
            np.testing.assert_allclose(st["conc"][0], ref.conc[:len(h.conc)], rtol=1e-11, atol=0)
            np.testing.assert_allclose(st["vm"][0], ref.vm, rtol=1e-11, atol=0)
        else:
            np.testing.assert_array_equal(st["conc"][0], ref.conc[:len(h.conc)])
            np.testing.assert_array_equal(st["vm"][0], ref.vm)
            np.testing.assert_array_equal(st["chip"][0], ref.chip)
    eng.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(PROGRAMS))
def test_engine_mixed_close_to_oracle(oracle, gpu_engine, name):
    """Mixed form: concentrations stay FP64; Vm within 1e-9 V, conc within
    1e-9 relative of the FP64 oracle after 1,000 steps."""
    h = build(name)
    eng = gpu_engine.Engine([h], precision=gpu_engine.PREC_MIXED)
    ref = oracle.Solver(h)
    eng.run(1000)
    ref.run(1000)
    st = eng.get_state()
    np.testing.assert_allclose(st["vm"][0], ref.vm, rtol=0, atol=1e-9)
    np.testing.assert_allclose(st["conc"][0], ref.conc[:len(h.conc)], rtol=1e-9, atol=0)
    eng.close()


@pytest.mark.gpu
def test_many_neurons_batched(oracle, gpu_engine):
    """64 copies of each program with perturbed initial Vm and conc in one
    batch: tiles of 32 neurons run the pool programs lane by lane."""
    hs, refs = [], []
    rng = np.random.default_rng(7)
    for name in sorted(PROGRAMS):
        for k in range(64):
            h = build(name)
            h.vm = h.vm + rng.uniform(-2e-3, 2e-3, len(h.vm))
            h.conc = np.asarray(h.conc) * rng.uniform(0.9, 1.1, len(h.conc))
            hs.append(h)
    eng = gpu_engine.Engine(hs)
    eng.run(300)
    st = eng.get_state()
    for i in range(0, len(hs), 17):
        ref = oracle.Solver(hs[i])
        ref.run(300)
        np.testing.assert_allclose(st["conc"][i], ref.conc[:len(hs[i].conc)], rtol=1e-11, atol=0)
        np.testing.assert_allclose(st["vm"][i], ref.vm, rtol=1e-11, atol=0)
    eng.close()
