"""Opcode coverage: hand-assembled compartment programs (tests/opprograms.py)
through the GPU engine (specialised and interpreted paths, FP64 and mixed)
against the reference's own step code, run once into the committed fixture
tests/golden/ref_opcodes.npz (tests/golden/make_golden.py), and against the
CPU oracle. Programs without libm calls must match bit for bit in FP64;
programs using exp/log (GHK, Nernst, Mg block) compare within 1e-12
relative, the distance between the CPU's libm and CUDA's math library."""
import os

import numpy as np
import pytest

import opprograms as P

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "ref_opcodes.npz")


def _compare(a, b, libm, tag=""):
    if libm:
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-18, err_msg=tag)
    else:
        np.testing.assert_array_equal(a, b, err_msg=tag)


@pytest.fixture(scope="module")
def ref_states():
    return np.load(FIXTURE, allow_pickle=False)


@pytest.mark.parametrize("jit", [True, False, 2, 3])
@pytest.mark.parametrize("name", sorted(P.PROGRAMS))
def test_program_fp64(oracle, gpu_engine, ref_states, name, jit):
    for mode in P.MODES:
        tag = P.mode_tag(name, *mode)
        h = P.from_fixture(ref_states, tag)        # the exact inputs the reference stepped
        libm = bool(ref_states[tag + "/libm"])
        eng = gpu_engine.Engine([h], jit=jit)
        eng.enable_givals(True)
        eng.run(P.NSTEPS)
        st = eng.get_state()
        giv = eng.givals()[0]
        # the reference's own step code (fixture)
        _compare(st["vm"][0], ref_states[tag + "/vm"], libm, tag)
        _compare(st["chip"][0], ref_states[tag + "/chip"], libm, tag)
        _compare(giv, ref_states[tag + "/givals"], libm, tag)
        if len(h.conc):
            _compare(st["conc"][0], ref_states[tag + "/conc"], libm, tag)
        keep = np.ones(len(h.ops), bool)
        keep[P.syn_countdown_words(h.ops)] = False
        np.testing.assert_array_equal(st["ops"][0][keep], ref_states[tag + "/ops"][keep], err_msg=tag)
        # the oracle restatement, run here
        ref = oracle.Solver(h)
        ref.run(P.NSTEPS)
        _compare(st["vm"][0], ref.vm, libm, tag)
        _compare(st["chip"][0], ref.chip, libm, tag)
        if len(h.conc):
            _compare(st["conc"][0], ref.conc[:len(h.conc)], libm, tag)
        _compare(giv, ref.givals, libm, tag)
        eng.close()


@pytest.mark.parametrize("name", sorted(P.PROGRAMS))
def test_program_mixed(oracle, gpu_engine, ref_states, name):
    tag = P.mode_tag(name, *P.MODES[0])
    h = P.from_fixture(ref_states, tag)
    eng = gpu_engine.Engine([h], precision=gpu_engine.PREC_MIXED)
    eng.run(P.NSTEPS)
    np.testing.assert_allclose(eng.vm(), ref_states[tag + "/vm"], rtol=0, atol=1e-9)
    ref = oracle.Solver(h)
    ref.run(P.NSTEPS)
    np.testing.assert_allclose(eng.vm(), ref.vm, rtol=0, atol=1e-9)
    eng.close()
