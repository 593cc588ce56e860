"""Symmetric compartments: the elimination program the reference's SETUP emits
for them (COPY_ARRAY, FASTSIBARRAY_ELIM, SIBARRAY_ELIM, hines_init.c:361-1273)
run by the engine as written (hines_solve.c:140-296).

Fixtures (tests/golden/make_symcompt.py): branched cells whose funcs[] /
ravals[] / diagonal terms come from the reference's own h_funcs_init, and
their state after 300 steps of the reference's own step code.

* CPU: the oracle reproduces the reference's trajectories bit for bit; the
  SETUP restatement (gbhsolve.model) reproduces the reference's asymmetric
  program for the same cells; the decoder accepts the programs (one neuron
  per solver) and rejects one with an index out of range.
* GPU: FP64 engine bit for bit against the reference's trajectories, alone
  and batched with tree-shaped solvers under every kernel form; mixed
  precision within 1e-6 V; the differentiated form refuses them.
"""
import os
import sys
from types import SimpleNamespace

import numpy as np
import pytest

from gbhsolve import model

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _load():
    return np.load(os.path.join(GOLDEN, "symcompt.npz"), allow_pickle=False)


def _case(d, name):
    g = lambda k: d[name + "/" + k]  # noqa: E731
    t = lambda k: d[name + "/" + k] if name + "/" + k in d.files else d["shared/" + k]  # noqa: E731
    sc = g("scalars")
    return SimpleNamespace(
        ncompts=int(sc[0]), ops=g("ops"), chip=g("chip").copy(), funcs=g("funcs"), ravals=g("ravals").copy(),
        vm=g("vm").copy(), givals=g("givals"), ncols=int(sc[1]), xdivs=int(sc[2]), xmin=float(sc[3]),
        invdx=float(sc[4]), tablist=t("tablist"), xvals=t("xvals"), ydivs=int(sc[5]),
        ymin=float(sc[6]), invdy=float(sc[7]), yvals=t("yvals"), stablist=g("stablist"), conc=g("conc"),
        concops=g("concops"), concchip=g("concchip"), childops=g("childops"), childchips=g("childchips"),
        dt=float(sc[8]), crank=int(sc[9]), chanmode=int(sc[10]), calcmode=int(sc[11]),
        method=11 if int(sc[9]) else 10)


def _names(d):
    return [str(x) for x in d["names"]]


def _cases_module():
    sys.path.insert(0, GOLDEN)
    try:
        import make_symcompt
    finally:
        sys.path.remove(GOLDEN)
    return make_symcompt


def test_fixtures_carry_symmetric_tokens():
    d = _load()
    assert len(_names(d)) == 7
    for name in _names(d):
        toks = set(int(t) for t in d[name + "/funcs"])
        assert {3, 4, 5} <= toks, name


def test_oracle_matches_reference_trajectories(oracle):
    d = _load()
    for name in _names(d):
        s = oracle.Solver(_case(d, name))
        s.run(int(d[name + "/nsteps"]))
        np.testing.assert_array_equal(s.vm, d[name + "/vm_ref"], err_msg=name)
        np.testing.assert_array_equal(s.chip, d[name + "/chip_ref"], err_msg=name)


def test_setup_restatement_matches_reference_asymmetric_program():
    """gbhsolve.model's h_funcs_init restatement against the reference's own
    setup on the same cells (asymmetric compartments)."""
    d = _load()
    mk = _cases_module()
    for name, m, _ in mk.cases():
        np.testing.assert_array_equal([c.parent for c in m.compartments], d[name + "/parents"])
        h = model.build(m)
        np.testing.assert_array_equal(h.funcs, d[name + "/asym_funcs"], err_msg=name)
        np.testing.assert_array_equal(h.ravals, d[name + "/asym_ravals"], err_msg=name)
        n = h.ncompts
        diag = [h.chip[len(h.chip) - 1 if i == n - 1 else h.compchips[i + 1] - 1] for i in range(n)]
        np.testing.assert_array_equal(diag, d[name + "/asym_diag"], err_msg=name)
        # the symmetric fixture is the same cell with the symmetric program
        np.testing.assert_array_equal(h.ops, d[name + "/ops"], err_msg=name)


def test_decoder_accepts_symmetric_programs():
    from gbhsolve import engine
    d = _load()
    hs = [_case(d, n) for n in _names(d)]
    nn, nt = engine.validate(hs)
    assert nn == len(hs)   # one neuron per solver, whatever its tree count
    assert nt == len(hs)


def test_decoder_rejects_out_of_range_sibling_index():
    from gbhsolve import engine
    d = _load()
    h = _case(d, "sym_star2x3_euler")
    f = h.funcs.copy()
    k = int(np.nonzero(f == 5)[0][0])    # first SIBARRAY_ELIM: operands are ravals indices
    f[k + 2] = len(h.ravals) + 7
    h.funcs = f
    with pytest.raises(engine.EngineError) as ei:
        engine.validate([h])
    assert ei.value.args and "range" in str(ei.value)


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [True, False])
def test_engine_fp64_matches_reference_trajectories(gpu_engine, jit):
    d = _load()
    for name in _names(d):
        h = _case(d, name)
        eng = gpu_engine.Engine([h], jit=jit, steps_per_launch=37)
        eng.run(int(d[name + "/nsteps"]))
        st = eng.get_state()
        np.testing.assert_array_equal(st["vm"][0], d[name + "/vm_ref"], err_msg=name)
        np.testing.assert_array_equal(st["chip"][0], d[name + "/chip_ref"], err_msg=name)
        eng.close()


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [True, False, 2, 3])
def test_engine_batched_with_trees(oracle, gpu_engine, jit):
    """Symmetric solvers (interpreted) beside tree-shaped ones (specialised
    where the form allows), several copies each, in one engine."""
    from gbhsolve import configs
    d = _load()
    sym = [_case(d, n) for n in _names(d)] * 6
    trees = [model.build(m) for m in configs.random_trees(40, size_range=(8, 40), seed=5)]
    hs = sym[:18] + trees + sym[18:]
    eng = gpu_engine.Engine(hs, jit=jit, steps_per_launch=50)
    eng.run(200)
    st = eng.get_state()
    for i in (0, 3, 9, 17, 18, 30, 57, 58, 62, 74):
        s = oracle.Solver(hs[i])
        s.run(200)
        np.testing.assert_array_equal(st["vm"][i], s.vm, err_msg=str(i))
        np.testing.assert_array_equal(st["chip"][i], s.chip, err_msg=str(i))
    eng.close()


@pytest.mark.gpu
def test_engine_mixed_within_tolerance(oracle, gpu_engine):
    """Mixed precision (double-float gate math, FP64 elimination): |dVm| <= 1e-6 V."""
    d = _load()
    hs = [_case(d, n) for n in _names(d)] * 3
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_MIXED)
    eng.run(300)
    st = eng.get_state()
    for i, name in enumerate(_names(d)):
        ref = oracle.Solver(hs[i])
        ref.run(300)
        err = np.max(np.abs(st["vm"][i] - ref.vm))
        assert err <= 1e-6, (name, err)
    eng.close()


@pytest.mark.gpu
def test_gradient_refuses_symmetric(gpu_engine):
    d = _load()
    h = _case(d, "sym_star2x3_euler")
    eng = gpu_engine.Engine([h], wide_min=-1)
    trace = np.zeros((10, 1))
    with pytest.raises(RuntimeError):
        eng.loss_gradient(10, [0], [0], trace)
    eng.close()


def test_symmetric_types_are_not_specialised():
    """The code generator declines symmetric-compartment tile types (they run
    on the interpreting kernels); the same cell as asymmetric compartments
    is specialised."""
    from gbhsolve import engine
    d = _load()
    assert engine.jit_source([_case(d, "sym_star2x3_euler")]) == ""
    mk = _cases_module()
    m = [c for c in mk.cases() if c[0] == "sym_star2x3_euler"][0][1]
    assert engine.jit_source([model.build(m)]) != ""


@pytest.mark.parametrize("damage", ["truncate", "extra_set", "bad_row", "odd_row"])
def test_decoder_rejects_malformed_symmetric_programs(damage):
    """A symmetric program is checked as it is decoded: it must end both
    passes on the right rows, and every row operand must be an even results
    index inside the solver."""
    from gbhsolve import engine
    d = _load()
    h = _case(d, "sym_star2x3_euler")
    f = [int(x) for x in h.funcs]
    fin = 0                                   # walk the forward pass to its FINISH
    while f[fin] != 7:
        fin += {0: 2, 1: 1, 2: 1, 3: 2, 4: 2, 5: 3}[f[fin]]
    if damage == "truncate":
        f = f[:fin - 3]
    elif damage == "extra_set":
        f.insert(fin, 1)                      # one row too many
    else:
        # walk the backward pass token by token to its last SIBARRAY_ELIM
        i, k = fin + 1, None
        while f[i] != 7:
            if f[i] == 5:
                k = i
            i += {0: 2, 6: 1, 5: 3}[f[i]]
        f[k + 2] = 2 * h.ncompts if damage == "bad_row" else f[k + 2] + 1
    h.funcs = np.array(f, np.int32)
    with pytest.raises(engine.EngineError) as ei:
        engine.validate([h])
    assert ei.value.code == -3
