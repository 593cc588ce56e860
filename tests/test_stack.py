"""Stack elimination (k_stack, k_stack_mixed): 32 neurons of many
compartments per warp, one per lane, whose rows are a post-order of their
trees (the Hines numbering of do_hnum, hines_init.c:317-345). The forward
elimination runs fused with the channel phase and keeps pending children's
contributions on a per-lane stack; back substitution reads each row's
(rhs, diagonal) from a column in global memory. FP64 results equal the
oracle (the reference's sequential step) bit for bit; the mixed form stays
within 1e-9 V of it. A tree numbered in another order (not a post-order)
falls back to the interpreter's shared-memory columns."""
import numpy as np
import pytest

import ophelpers as A
from gbhsolve import configs, model

pytestmark = pytest.mark.gpu


def _trees(method, seed=9):
    # three sizes, 40 neurons each: full and partial tiles of one program
    hs = []
    for k, n in enumerate((48, 130, 255)):
        hs += [model.build(m) for m in configs.random_trees(40, size_range=(n, n), seed=seed + k, method=method)]
    return hs


def _oracle_run(oracle, h, n):
    s = oracle.Solver(h)
    s.run(n)
    return s


@pytest.mark.parametrize("jit", [False, True])
@pytest.mark.parametrize("method", [model.BEULER, model.CRANK])
def test_random_trees_stack_fp64(oracle, gpu_engine, method, jit):
    hs = _trees(method)
    eng = gpu_engine.Engine(hs, wide_min=-1, jit=jit, steps_per_launch=50)
    st = eng.stats()
    assert st.wide_tiles == 0
    if not jit:
        assert st.stack_tiles == st.tiles == 6
    eng.enable_givals(True)
    eng.run(200)
    s = eng.get_state()
    giv = eng.givals()
    for i in list(range(0, len(hs), 7)) + [39, 79, 119]:
        ref = _oracle_run(oracle, hs[i], 200)
        np.testing.assert_array_equal(s["vm"][i], ref.vm)
        np.testing.assert_array_equal(s["chip"][i], ref.chip)
        np.testing.assert_array_equal(s["conc"][i], ref.conc[:len(hs[i].conc)])
        np.testing.assert_array_equal(giv[i], ref.givals)
    eng.close()


def test_random_trees_stack_mixed(oracle, gpu_engine):
    hs = _trees(model.BEULER, seed=21)
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_MIXED, wide_min=-1, jit=False)
    assert eng.stats().stack_tiles == 6
    worst = 0.0
    refs = [oracle.Solver(hs[i]) for i in range(0, len(hs), 5)]
    for _ in range(3):
        eng.run(100)
        for r in refs:
            r.run(100)
        vm = eng.get_state()["vm"]
        worst = max(worst, max(float(np.max(np.abs(vm[i] - r.vm))) for i, r in zip(range(0, len(hs), 5), refs)))
    assert worst <= 1e-9, worst
    eng.close()


def test_stack_equals_wide_and_interpreter(gpu_engine):
    """One batch of uneven trees three ways -- wide tiles (the smaller trees
    on stack tiles), stack elimination throughout, specialised kernels where
    they apply -- bit-identical in FP64."""
    hs = [model.build(m) for m in configs.random_trees(96, size_range=(8, 200), seed=23)]
    a = gpu_engine.Engine(hs, wide_min=32, jit=False)
    b = gpu_engine.Engine(hs, wide_min=-1, jit=False)
    c = gpu_engine.Engine(hs, wide_min=-1, jit=True)
    assert a.stats().wide_tiles > 0 and b.stats().wide_tiles == 0 and b.stats().stack_tiles > 0
    for e in (a, b, c):
        e.run(300)
    np.testing.assert_array_equal(a.vm(), b.vm())
    np.testing.assert_array_equal(a.vm(), c.vm())
    for e in (a, b, c):
        e.close()


def _level_numbered_tree(levels=6):
    """A complete binary tree with its rows numbered level by level from the
    leaves (children still before parents, but no subtree contiguous)."""
    n = 2 ** levels - 1
    parents = []
    start, width = 0, 2 ** (levels - 1)
    while width > 1:
        for i in range(width):
            parents.append(start + width + i // 2)
        start += width
        width //= 2
    parents.append(-1)
    assert len(parents) == n
    return parents


def test_non_postorder_tree_falls_back(oracle, gpu_engine):
    parents = _level_numbered_tree()
    n = len(parents)
    dt = 2e-5
    comps = []
    for i in range(n):
        c = A.Compt(-0.065 / 3e8, 1e-10 if i == n - 1 else 0.0, dt / 1e-11, 1.0 + dt / (1e-11 * 3e8), 3e8,
                    -0.06 + 1e-4 * i)
        if i == n - 1:
            c.op(A.NEWVOLT).op(A.CHAN_EK, chips=[0.05, 1e-8]).op(A.IPOL1V, 0, 3, chips=[0.1])
            c.op(A.IPOL1V, 2, 1, chips=[0.6]).op(A.ADD_CURR, giv=3)
        comps.append(c)
    h = A.solver(comps, A.tables(12, 40), dt=dt, parents=parents)
    # coupling coefficients small enough for a diagonally dominant matrix
    h.ravals = -1e-3 * (1.0 + 0.1 * np.sin(np.arange(len(h.ravals))))
    eng = gpu_engine.Engine([h] * 33, wide_min=-1, jit=False)
    assert eng.stats().stack_tiles == 0          # not a post-order: the interpreter's columns
    eng.run(300)
    ref = _oracle_run(oracle, h, 300)
    vm = eng.get_state()["vm"]
    np.testing.assert_array_equal(vm[0], ref.vm)
    np.testing.assert_array_equal(vm[32], ref.vm)
    eng.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_static_rows_follow_inputs_and_state_between_launches(oracle, gpu_engine, prec):
    """Passive rows below every channel keep their diagonal terms in a launch
    after its first step; inputs (the soma's and a dendrite's inject) and
    state writes (a dendrite's Em/Rm term) between launches must reach them."""
    hs = _trees(model.BEULER, seed=41)
    p = gpu_engine.PREC_FP64 if prec == "fp64" else gpu_engine.PREC_MIXED
    eng = gpu_engine.Engine(hs, precision=p, wide_min=-1, jit=False, steps_per_launch=20)
    assert eng.stats().stack_tiles == eng.stats().tiles
    rows = []
    for i, h in enumerate(hs):
        rows.append((i, int(h.compchips[h.ncompts - 1]) + 1))      # the soma's inject
        rows.append((i, int(h.compchips[3]) + 1))                  # a dendrite's inject
    eng.register_inputs(np.array([r[0] for r in rows], np.int32), np.array([r[1] for r in rows]))
    refs = [oracle.Solver(h) for h in hs]
    rng = np.random.default_rng(42)
    worst = 0.0
    for k in range(6):
        v = rng.uniform(0.0, 1e-9, size=len(rows))
        eng.set_inputs_async(v, 0)
        for (i, c), x in zip(rows, v):
            refs[i].chip[c] = x
        if k == 3:                                  # a state write between launches
            st = eng.get_state()
            for i, h in enumerate(hs):
                c = int(h.compchips[5])             # row 5's Em/Rm term
                st["chip"][i][c] *= 1.25
                refs[i].chip[c] = st["chip"][i][c]
            eng.set_state(chip=st["chip"])
        eng.run(20)
        for r in refs:
            r.run(20)
        vm = eng.get_state()["vm"]
        for i, r in enumerate(refs):
            if prec == "fp64":
                np.testing.assert_array_equal(vm[i], r.vm)
            else:
                worst = max(worst, float(np.max(np.abs(vm[i] - r.vm))))
    assert worst <= 1e-9, worst
    eng.close()


def _three_child_trees(n, size, seed):
    """Random trees whose root gets a third child (a subtree moved under it),
    so the forward sweep pops two stacked children at one row."""
    ms = configs.random_trees(n, size_range=(size, size), seed=seed)
    for m in ms:
        comps = m.compartments
        k = next(i for i in range(len(comps) - 1, 0, -1) if comps[i].parent not in (-1, 0))
        comps[k].parent = 0
    return [model.build(m) for m in ms]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_stack_rows_with_three_children(oracle, gpu_engine, prec):
    """A type whose rows pop more than one stacked child takes the general
    forward sweep (a loop over the popped entries, a running stack top) on
    every step, including the static rows' rhs-only steps."""
    hs = _three_child_trees(40, 64, seed=51)
    p = gpu_engine.PREC_FP64 if prec == "fp64" else gpu_engine.PREC_MIXED
    eng = gpu_engine.Engine(hs, precision=p, wide_min=-1, jit=False, steps_per_launch=25)
    assert eng.stats().stack_tiles == eng.stats().tiles
    eng.run(100)
    vm = eng.get_state()["vm"]
    for i in range(0, len(hs), 3):
        ref = _oracle_run(oracle, hs[i], 100)
        if prec == "fp64":
            np.testing.assert_array_equal(vm[i], ref.vm)
        else:
            assert float(np.max(np.abs(vm[i] - ref.vm))) <= 1e-9
    eng.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kept_factors_across_launches(oracle, gpu_engine, prec):
    """The static rows' kept factors outlive a launch. One-step launches (the
    hsolve-level ABI's use) take the fast path from the second launch on; a
    state write of a static row's diagonal term, and an input that sets one
    every launch, make the next launch redo them."""
    hs = _trees(model.BEULER, seed=61)
    p = gpu_engine.PREC_FP64 if prec == "fp64" else gpu_engine.PREC_MIXED
    eng = gpu_engine.Engine(hs, precision=p, wide_min=-1, jit=False, steps_per_launch=1)
    refs = [oracle.Solver(h) for h in hs]
    worst = 0.0

    def check():
        nonlocal worst
        vm = eng.get_state()["vm"]
        for i, r in enumerate(refs):
            if prec == "fp64":
                np.testing.assert_array_equal(vm[i], r.vm)
            else:
                worst = max(worst, float(np.max(np.abs(vm[i] - r.vm))))

    for _ in range(40):                           # 40 one-step launches
        eng.run(1)
    for r in refs:
        r.run(40)
    check()
    st = eng.get_state()                          # row 5's diagonal term, written between launches
    for i, h in enumerate(hs):
        c = int(h.compchips[5]) + 3
        st["chip"][i][c] *= 1.02
        refs[i].chip[c] = st["chip"][i][c]
    eng.set_state(chip=st["chip"])
    for _ in range(20):
        eng.run(1)
    for r in refs:
        r.run(20)
    check()
    # an input that sets row 3's diagonal term before every launch
    rows = [(i, int(h.compchips[3]) + 3) for i, h in enumerate(hs)]
    eng.register_inputs(np.array([r[0] for r in rows], np.int32), np.array([r[1] for r in rows]))
    base = np.array([refs[i].chip[c] for i, c in rows])
    for k in range(10):
        v = base * (1.0 + 0.01 * (k % 3))
        eng.set_inputs_async(v, 0)
        for (i, c), x in zip(rows, v):
            refs[i].chip[c] = x
        eng.run(3)
        for r in refs:
            r.run(3)
    check()
    assert worst <= 1e-9, worst
    eng.close()
