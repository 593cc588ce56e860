"""h_in_msgs input kinds (hines_msgs.c:351-405) through
gbh_register_inputs_typed: INJECT (set), SYN2 activation (added when above
VTINY, scaled by stablist[nop+3] and by dt for ACTIVATION messages), FLUX
(sets a concentration's flux). The oracle gets the same inputs applied to its
arrays in registration order before each step; states must be equal bit for
bit."""
import numpy as np
import pytest

import ophelpers as A

pytestmark = pytest.mark.gpu
DT = 2e-5


def _model():
    rng = np.random.default_rng(5)
    cov0, _, conc = A.diffusion_system(rng, 4, dt=DT, crank=True)
    c = A.Compt(emrm=-0.065 / 1e9, inject=1e-10, tbyc=DT / 1e-11, diag=1.0 + DT / 1e-11 / 1e9, rm=1e9, vm0=-0.06)
    # chip layout: 0 Em/Rm, 1 inject, 2 Ek, 3 gmax, 4 X, 5 Y, 6 Ek(Ca), 7 gmax(Ca), 8 gate, 9 tbyc, 10 diag
    c.op(A.CHAN_EK, chips=[0.0, 2e-9]).op(A.SYN2, 0, -1, 1, chips=[0.0, 0.0], giv=3)
    c.op(A.NEWVOLT).op(A.CONC_VAL, 0).op(A.CHAN_EK, chips=[0.12, 3e-11]).op(A.IPOL1V, 0, 4, chips=[0.3])
    c.op(A.ADD_CURR, giv=3).op(A.FLUX)
    xc2, yc1, yc2, xc1 = 0.99, 9.5e-5, 0.98, 9.9e-5
    ops = [A.FCONC, 0, A.FLUXCONC, A.CONC, 2, A.FLUXCONC, A.MMPUMP, A.LCONC]
    chips = [0.0, 5e5, 1e-9, 2e5, 1e-6, 1e-3]
    diff = dict(dconc=[0], nshells=[4], nshrows=[1], nshfix=[0], fbufval=[0], covals0=cov0, bufvals=[])
    h = A.solver([c], A.tables(12, 40, seed=3), dt=DT, crank=True, stablist=[xc2, yc1, yc2, xc1 / DT],
                 conc=conc, concops=ops, concchip=chips, diff=diff)
    return h, xc1 / DT


def test_typed_inputs_equal_oracle(oracle, gpu_engine):
    h, s3 = _model()
    eng = gpu_engine.Engine([h], steps_per_launch=1)
    # inject (set), two activation messages into the same synchan X (added in
    # order; the second one as ACTIVATION: times dt), a flux into shell 2
    kinds = np.array([gpu_engine.IN_SET, gpu_engine.IN_ADD, gpu_engine.IN_ADD, gpu_engine.IN_FLUX])
    index = np.array([1, 4, 4, 2])
    sa = np.array([1.0, s3, s3, 1.0])
    sb = np.array([1.0, 1.0, DT, 1.0])
    eng.register_inputs(np.zeros(4, np.int32), index, kind=kinds, sa=sa, sb=sb)
    ref = oracle.Solver(h)
    rng = np.random.default_rng(11)
    for k in range(400):
        v = np.array([rng.uniform(0, 3e-10), rng.choice([0.0, 1e-11, rng.uniform(0, 2.0)]),
                      rng.uniform(0, 50.0), rng.uniform(-1e-13, 1e-12)])
        eng.set_inputs_async(v, 0)
        eng.run(1)
        # h_in_msgs on the oracle's arrays, list order
        ref.chip[1] = v[0]
        for j in (1, 2):
            if v[j] > 1e-10:
                ref.chip[4] += v[j] * sa[j] * sb[j]
        ref.flux[2] = v[3]
        ref.run(1)
    st = eng.get_state()
    np.testing.assert_array_equal(st["chip"][0], ref.chip)
    np.testing.assert_array_equal(st["vm"][0], ref.vm)
    np.testing.assert_array_equal(st["conc"][0], ref.conc[:len(h.conc)])
    assert ref.chip[4] != 0.0
    eng.close()


def test_run_io_with_typed_inputs(oracle, gpu_engine):
    """The same inputs streamed with gbh_run_io (block of 7 steps)."""
    h, s3 = _model()
    eng = gpu_engine.Engine([h], steps_per_launch=1)
    kinds = np.array([gpu_engine.IN_SET, gpu_engine.IN_ADD, gpu_engine.IN_FLUX])
    eng.register_inputs(np.zeros(3, np.int32), np.array([1, 4, 2]), kind=kinds, sa=np.array([1.0, s3, 1.0]))
    eng.register_outputs(np.zeros(1, np.int32), np.zeros(1, np.int32))
    n = 100
    rng = np.random.default_rng(12)
    vin = np.stack([rng.uniform(0, 3e-10, n), rng.choice([0.0, 0.5, 1.5], n), rng.uniform(0, 1e-12, n)], axis=1)
    vout = np.empty((n, 1))
    eng.run_io(np.ascontiguousarray(vin), vout, n, block=7)
    ref = oracle.Solver(h)
    for k in range(n):
        ref.chip[1] = vin[k, 0]
        if vin[k, 1] > 1e-10:
            ref.chip[4] += vin[k, 1] * s3 * 1.0
        ref.flux[2] = vin[k, 2]
        ref.run(1)
        assert vout[k, 0] == ref.vm[0], k
    np.testing.assert_array_equal(eng.get_state()["conc"][0], ref.conc[:len(h.conc)])
    eng.close()
