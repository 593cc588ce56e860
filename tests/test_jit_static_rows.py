"""Specialised kernels (gbh_jit, the register form of a shared tree) keep the
factors of the passive rows below the first compartment with channels -- the
rhs term K, T = A/D' and D' (FP64) or 1/D' (mixed) -- across steps and
launches. FP64 results stay equal to the oracle (the reference's sequential
step) bit for bit through multi-step and one-step launches, a state write of
a static row's fields between launches, per-step inputs on a static row's
inject (applied inside the kernel by gbh_run_io, and between launches) and an
input on a static row's diagonal term; the mixed form stays within 1e-9 V."""
import numpy as np
import pytest

from gbhsolve import configs, model

pytestmark = pytest.mark.gpu


def _cables(n=80, seed=7, method=model.BEULER):
    # passive dendrites (no gk_dend): rows 0-14 static, the soma (row 15) active
    return [model.build(m) for m in configs.cables(n, seed=seed, method=method, per_neuron_solvers=True)]


def _check(eng, refs, prec, worst):
    vm = eng.get_state()["vm"]
    for i, r in enumerate(refs):
        if prec == "fp64":
            np.testing.assert_array_equal(vm[i], r.vm)
        else:
            worst[0] = max(worst[0], float(np.max(np.abs(vm[i] - r.vm))))


@pytest.mark.parametrize("method", [model.BEULER, model.CRANK])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kept_factors_in_specialised_kernels(oracle, gpu_engine, prec, method):
    hs = _cables(method=method)
    p = gpu_engine.PREC_FP64 if prec == "fp64" else gpu_engine.PREC_MIXED
    assert "kept factors" in gpu_engine.jit_source(hs[:1], p, 0, 0)
    eng = gpu_engine.Engine(hs, precision=p, wide_min=-1, jit=True, steps_per_launch=16)
    assert eng.stats().jit_kernels >= 1
    refs = [oracle.Solver(h) for h in hs]
    worst = [0.0]

    def step_both(n):
        eng.run(n)
        for r in refs:
            r.run(n)

    step_both(40)                                  # launches of 16, 16 and 8 steps
    _check(eng, refs, prec, worst)
    st = eng.get_state()                           # row 5's Em/Rm term, written between launches
    for i, h in enumerate(hs):
        c = int(h.compchips[5])
        st["chip"][i][c] *= 1.25
        refs[i].chip[c] = st["chip"][i][c]
    eng.set_state(chip=st["chip"])
    step_both(20)
    _check(eng, refs, prec, worst)
    # per-step inputs on the soma's and row 3's inject (a static row's rhs)
    rows = []
    for i, h in enumerate(hs):
        rows.append((i, int(h.compchips[h.ncompts - 1]) + 1))
        rows.append((i, int(h.compchips[3]) + 1))
    eng.register_inputs(np.array([r[0] for r in rows], np.int32), np.array([r[1] for r in rows]))
    rng = np.random.default_rng(8)
    nsteps = 48
    stim = np.ascontiguousarray(rng.uniform(0.0, 5e-10, size=(nsteps, len(rows))))
    eng.run_io(stim, None, nsteps, 16)
    for k in range(nsteps):
        for (i, c), x in zip(rows, stim[k]):
            refs[i].chip[c] = x
        for r in refs:
            r.run(1)
    _check(eng, refs, prec, worst)
    for k in range(5):                             # the same inputs set between launches
        v = stim[k]
        eng.set_inputs_async(v, 0)
        for (i, c), x in zip(rows, v):
            refs[i].chip[c] = x
        step_both(7)
    _check(eng, refs, prec, worst)
    assert worst[0] <= 1e-9, worst[0]
    eng.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_specialised_static_rows_one_step_launches_and_diagonal_inputs(oracle, gpu_engine, prec):
    """One-step launches (the hsolve-level ABI's use) take the kept factors
    from the second launch on; an input that sets a static row's diagonal
    term makes every step a full one."""
    hs = _cables(48, seed=9)
    p = gpu_engine.PREC_FP64 if prec == "fp64" else gpu_engine.PREC_MIXED
    eng = gpu_engine.Engine(hs, precision=p, wide_min=-1, jit=True, steps_per_launch=1)
    refs = [oracle.Solver(h) for h in hs]
    worst = [0.0]
    for _ in range(30):
        eng.run(1)
    for r in refs:
        r.run(30)
    _check(eng, refs, prec, worst)
    rows = [(i, int(h.compchips[3]) + 3) for i, h in enumerate(hs)]   # row 3's diagonal term
    eng.register_inputs(np.array([r[0] for r in rows], np.int32), np.array([r[1] for r in rows]))
    base = np.array([refs[i].chip[c] for i, c in rows])
    for k in range(8):
        v = base * (1.0 + 0.01 * (k % 3))
        eng.set_inputs_async(v, 0)
        for (i, c), x in zip(rows, v):
            refs[i].chip[c] = x
        eng.run(3)
        for r in refs:
            r.run(3)
    _check(eng, refs, prec, worst)
    assert worst[0] <= 1e-9, worst[0]
    eng.close()
