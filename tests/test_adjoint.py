"""Differentiated form: gbh_loss_gradient (hand-written adjoint kernels).

Loss = sum over steps and target rows of (Vm after the step - trace)^2.
Checks:
  * the CPU reference gradient (oracle/adjoint_ref.py, torch autograd of a
    restatement of the reference step) against central finite differences of
    the oracle (CPU, no GPU);
  * the engine's gradient with respect to every chip[], ravals[] and initial
    vm[] entry against the CPU reference gradient (relative 1e-9 of the
    array's largest entry): backward Euler and Crank-Nicolson, calcmode 0/1,
    chanmode 4/5, several targets per neuron, many solvers;
  * checkpoint interval invariance, loss value against the oracle, engine
    state untouched, unsupported programs rejected;
  * the config-4 workload shape (64-compartment random trees, 10,000 steps,
    checkpoints every 100) against central finite differences with
    h = 1e-6 relative on 64 sampled physical parameters (per-compartment
    gbar of Na, K and leak, per-neuron CM and RA), through the chain rule
    from the array gradient to the physical parameters.
The piecewise-linear gate tables make the loss piecewise smooth: a central
difference whose +-h interval straddles a table node of some lookup averages
two slopes. That bias is the finite-difference error, not the gradient's;
the tests bound it as stated at each assertion.
"""
import copy

import numpy as np
import pytest

from gbhsolve import configs, model

DT = 25e-6


def _trees(n, ncomp, seed, method=model.BEULER):
    trees, (na, k) = configs.grad_trees(n, ncomp=ncomp, seed=seed)
    hs = [model.build(t.model(na, k, dt=DT, method=method), exact=True) for t in trees]
    return trees, (na, k), hs


def _oracle_trace(oracle, hs, nsteps, rows_per_solver):
    """Target traces: Vm of the given rows after every step, from the oracle."""
    out = []
    for h, rows in zip(hs, rows_per_solver):
        s = oracle.Solver(h)
        tr = np.empty((nsteps, len(rows)))
        for n in range(nsteps):
            s.run(1)
            tr[n] = s.vm[rows]
        out.append(tr)
    return out


def _rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


FD_TOL = 1e-4


def fd_rule(oracle, tree, chans, j, g, nsteps, rows, trace, rel_h=1e-6):
    """Per-sample finite-difference rule for the gradient g of parameter j.

    Differences of the loss between two runs are formed from their traces,
    L(a) - L(b) = sum (a - b)(a + b - 2 target), which keeps the digits a
    difference of two 10,000-step sums would cancel. A central difference
    (h = rel_h x |p|) must agree with g within FD_TOL. If it does not:

    * the loss is piecewise smooth -- the gates interpolate tables linearly,
      so its slope jumps where a perturbation moves some compartment's Vm
      across a table node at some step. If the runs at p - h and p + h put
      some compartment in different table rows at some step, g is the slope
      on one side of the kink: the forward or the backward difference must
      agree with it within FD_TOL ("one-sided");
    * otherwise the difference may be below what the runs resolve: rounding
      in a spiking 10,000-step trajectory puts noise into every trace, and a
      parameter with a small effect on the soma moves the loss by little
      more than that. The spread between the forward and the backward
      difference at the same h -- O(h) for a smooth loss, O(1/h) for noise
      -- measures it. When that spread exceeds FD_TOL, the central
      difference is repeated at 10 h and 100 h (noise falls as 1/h, the
      truncation error of a central difference as h^2), without a table
      node in the interval; one of them with a spread within FD_TOL must
      agree with g within FD_TOL ("central at 10h" / "central at 100h").

    Returns (kind, rel err); kind "fail" when no rule holds."""
    na, k = chans
    v = tree.vector()
    target = np.asarray(trace, dtype=np.float64).reshape(int(nsteps), len(rows))
    runs = {}

    def run(delta):
        if delta not in runs:
            w = v.copy()
            w[j] += delta
            hh = model.build(tree.with_vector(w).model(na, k, dt=DT), exact=True)
            runs[delta] = oracle.Solver(hh).run_trace(nsteps, rows, table_rows=True)
        return runs[delta]

    def dloss(a, b):
        ta, tb = run(a)[0], run(b)[0]
        return float(np.sum((ta - tb) * (ta + tb - 2.0 * target)))

    def diffs(step):
        c = dloss(step, -step) / (2 * step)
        f = dloss(step, 0.0) / step
        b = dloss(0.0, -step) / step
        return c, f, b, not np.array_equal(run(step)[1], run(-step)[1])

    h0 = rel_h * abs(v[j])
    c, f, b, kink = diffs(h0)
    if _rel(c, g) <= FD_TOL:
        return "central", _rel(c, g)
    if kink:
        one = min(_rel(f, g), _rel(b, g))
        return ("one-sided" if one <= FD_TOL else "fail"), one
    if _rel(f, b) > FD_TOL:           # below the resolution of the runs at h
        for m in (10.0, 100.0):
            c2, f2, b2, kink2 = diffs(m * h0)
            if not kink2 and _rel(f2, b2) <= FD_TOL and _rel(c2, g) <= FD_TOL:
                return "central at %dh" % int(m), _rel(c2, g)
    return "fail", _rel(c, g)


# --------------------------------------------------------------------------
# CPU: the reference gradient itself
# --------------------------------------------------------------------------
@pytest.mark.parametrize("method", [model.BEULER, model.CRANK])
def test_cpu_reference_gradient_matches_oracle_fd(oracle, method):
    import adjoint_ref
    trees, (na, k), hs = _trees(1, 8, seed=7, method=method)
    h = hs[0]
    nsteps = 300
    rows = [h.ncompts - 1, 2]
    rng = np.random.default_rng(1)
    trace = -0.065 + 0.01 * rng.normal(size=(nsteps, 2))
    L, gc, gr, gv = adjoint_ref.loss_and_gradient(h, nsteps, rows, trace)
    assert _rel(L, oracle.Solver(h).run_loss(nsteps, rows, trace)) < 1e-13

    L0 = oracle.Solver(h).run_loss(nsteps, rows, trace)

    def fd(name, j, rel):
        """Central, forward and backward differences with step rel*|a_j|."""
        a = np.array(getattr(h, name), copy=True)
        step = rel * abs(a[j])
        out = []
        for sgn in (1.0, -1.0):
            hh = copy.copy(h)
            b = a.copy()
            b[j] += sgn * step
            setattr(hh, name, b)
            out.append(oracle.Solver(hh).run_loss(nsteps, rows, trace))
        return (out[0] - out[1]) / (2 * step), (out[0] - L0) / step, (L0 - out[1]) / step

    checked = 0
    for name, g in (("chip", gc), ("ravals", gr), ("vm", gv)):
        a = getattr(h, name)
        for j in range(0, len(a), max(1, len(a) // 10)):
            if a[j] == 0.0 or abs(g[j]) * abs(a[j]) < 1e-12 * L:
                continue
            # kinks bias large steps and roundoff small ones (entries with a
            # small gradient); where the evaluation point itself sits on a
            # table node (initial Vm = -0.065 V is one, within rounding) the
            # adjoint gives the slope on the side the lookup chose, which a
            # one-sided difference reproduces. The best of six steps x three
            # difference formulas must agree to 1e-5.
            err = min(_rel(d, g[j]) for r in (1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9) for d in fd(name, j, r))
            assert err < 1e-5, (name, j, g[j], err)
            checked += 1
    assert checked >= 15


# --------------------------------------------------------------------------
# GPU: engine gradient against the CPU reference gradient
# --------------------------------------------------------------------------
def _engine_vs_reference(oracle, gpu_engine, hs, rows_per_solver, nsteps, checkpoint_every=40):
    import adjoint_ref
    rng = np.random.default_rng(11)
    traces = [-0.065 + 0.02 * rng.normal(size=(nsteps, len(r))) for r in rows_per_solver]
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_FP64, wide_min=-1)
    solver = np.concatenate([np.full(len(r), i) for i, r in enumerate(rows_per_solver)])
    row = np.concatenate(rows_per_solver)
    trace = np.concatenate(traces, axis=1)
    L, dchip, drav, dvm = eng.loss_gradient(nsteps, solver, row, trace, checkpoint_every)
    b = eng.batch
    Lref = 0.0
    for i, h in enumerate(hs):
        l, gc, gr, gv = adjoint_ref.loss_and_gradient(h, nsteps, list(rows_per_solver[i]), traces[i])
        Lref += l
        for name, mine, ref, st in (("chip", dchip, gc, b.chip_start), ("ravals", drav, gr, b.ravals_start),
                                    ("vm", dvm, gv, b.vm_start)):
            m = mine[st[i]:st[i + 1]]
            scale = max(float(np.max(np.abs(ref))), 1e-300)
            err = float(np.max(np.abs(m - ref))) / scale
            assert err < 1e-9, (i, name, err)
    assert _rel(L, Lref) < 1e-12
    eng.close()
    return L


@pytest.mark.gpu
@pytest.mark.parametrize("method", [model.BEULER, model.CRANK])
def test_gradient_matches_cpu_reference(oracle, gpu_engine, method):
    trees, _, hs = _trees(3, 8, seed=21, method=method)
    rows = [[h.ncompts - 1] for h in hs]
    _engine_vs_reference(oracle, gpu_engine, hs, rows, 250)


@pytest.mark.gpu
def test_gradient_several_targets_per_neuron(oracle, gpu_engine):
    trees, _, hs = _trees(2, 10, seed=22)
    rows = [[h.ncompts - 1, 0, 3] for h in hs]
    _engine_vs_reference(oracle, gpu_engine, hs, rows, 200)


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["calcmode0", "chanmode5"])
def test_gradient_solver_modes(oracle, gpu_engine, variant):
    trees, _, hs = _trees(2, 8, seed=23)
    for h in hs:
        if variant == "calcmode0":
            h.calcmode = 0
        else:
            h.chanmode = 5
    rows = [[h.ncompts - 1] for h in hs]
    _engine_vs_reference(oracle, gpu_engine, hs, rows, 200)


@pytest.mark.gpu
def test_gradient_one_solver_many_trees(oracle, gpu_engine):
    """Several neurons in one hsolve (roots in list order)."""
    trees, (na, k) = configs.grad_trees(3, ncomp=6, seed=24)
    comps = []
    for t in trees:
        m = t.model(na, k, dt=DT)
        base = len(comps)
        for c in m.compartments:
            if c.parent >= 0:
                c.parent += base
        comps += m.compartments
    h = model.build(model.Model(comps, dt=DT, method=model.BEULER), exact=True)
    roots = [int(h.hnum[i]) for i, c in enumerate(comps) if c.parent < 0]
    _engine_vs_reference(oracle, gpu_engine, [h], [roots], 150)


@pytest.mark.gpu
def test_checkpoint_interval_invariance_and_state(oracle, gpu_engine):
    trees, _, hs = _trees(40, 16, seed=25)
    nsteps = 600
    rows = [[h.ncompts - 1] for h in hs]
    traces = _oracle_trace(oracle, _trees(40, 16, seed=26)[2], nsteps, rows)
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_FP64, wide_min=-1)
    solver = np.arange(len(hs))
    row = np.array([r[0] for r in rows])
    trace = np.concatenate(traces, axis=1)
    vm0 = eng.vm().copy()
    base = eng.loss_gradient(nsteps, solver, row, trace, 100)
    assert eng.stats().grad_kept_steps == 0
    # 0: every step's state kept in device memory, no segment recomputed
    for K in (1, 7, 600, 5000, 0):
        other = eng.loss_gradient(nsteps, solver, row, trace, K)
        assert eng.stats().grad_kept_steps == (1 if K == 0 else 0)
        assert other[0] == base[0]
        for a, b in zip(other[1:], base[1:]):
            assert np.array_equal(a, b), K
    # the engine state is untouched and the loss equals the oracle's
    assert np.array_equal(eng.vm(), vm0)
    Lo = sum(oracle.Solver(h).run_loss(nsteps, [r[0]], tr) for h, r, tr in zip(hs, rows, traces))
    assert _rel(base[0], Lo) < 1e-12
    eng.run(nsteps)
    orc = [oracle.Solver(h) for h in hs]
    for s in orc:
        s.run(nsteps)
    assert np.array_equal(eng.vm(), np.concatenate([s.vm for s in orc]))
    eng.close()


@pytest.mark.gpu
def test_unsupported_programs_rejected(gpu_engine):
    hs = [model.build(m) for m in configs.random_trees(2, size_range=(8, 12), seed=5)]   # Ca pools
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_FP64, wide_min=-1)
    with pytest.raises(RuntimeError, match="error -6"):
        eng.loss_gradient(10, [0], [hs[0].ncompts - 1], np.zeros(10))
    eng.close()
    trees, _, hs = _trees(2, 8, seed=27)
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_MIXED)
    with pytest.raises(RuntimeError, match="error -6"):
        eng.loss_gradient(10, [0], [hs[0].ncompts - 1], np.zeros(10))
    eng.close()
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_FP64, wide_min=-1)
    with pytest.raises(RuntimeError, match="error -1"):     # target row out of range
        eng.loss_gradient(10, [0], [999], np.zeros(10))
    with pytest.raises(RuntimeError, match="error -1"):     # repeated target
        eng.loss_gradient(10, [0, 0], [1, 1], np.zeros((10, 2)))
    eng.close()


@pytest.mark.gpu
def test_autograd_function_wrapper(oracle, gpu_engine):
    """The C ABI wrapped as a torch.autograd.Function (tests only): the
    gradient reaching leaf tensors through autograd equals the ABI's."""
    import torch

    trees, _, hs = _trees(4, 8, seed=28)
    nsteps = 120
    rows = np.array([h.ncompts - 1 for h in hs])
    trace = np.full((nsteps, len(hs)), -0.06)
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_FP64, wide_min=-1)
    b = eng.batch

    class SomaLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, chip, ravals, vm0):
            eng.set_state(vm=vm0.detach().numpy(), chip=chip.detach().numpy())
            L, dc, dr, dv = eng.loss_gradient(nsteps, np.arange(len(hs)), rows, trace, 30)
            ctx.save_for_backward(torch.from_numpy(dc[:len(b.chip)]), torch.from_numpy(dr[:len(b.ravals)]),
                                  torch.from_numpy(dv[:len(b.vm)]))
            return torch.tensor(L, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            dc, dr, dv = ctx.saved_tensors
            return gout * dc, gout * dr, gout * dv

    chip = torch.tensor(b.chip, dtype=torch.float64, requires_grad=True)
    rav = torch.tensor(b.ravals, dtype=torch.float64, requires_grad=True)
    vm0 = torch.tensor(b.vm, dtype=torch.float64, requires_grad=True)
    loss = 3.0 * SomaLoss.apply(chip, rav, vm0)
    loss.backward()
    L, dc, dr, dv = eng.loss_gradient(nsteps, np.arange(len(hs)), rows, trace, 30)
    assert np.array_equal(chip.grad.numpy(), 3.0 * dc[:len(b.chip)])
    assert np.array_equal(rav.grad.numpy(), 3.0 * dr[:len(b.ravals)])
    assert np.array_equal(vm0.grad.numpy(), 3.0 * dv[:len(b.vm)])
    eng.close()


# --------------------------------------------------------------------------
# GPU: config-4 shape against finite differences on physical parameters
# --------------------------------------------------------------------------
@pytest.mark.gpu
def test_config4_shape_physical_parameters_vs_fd(oracle, gpu_engine):
    n_neurons, ncomp, nsteps, K = 64, 64, 10000, 100
    trees, (na, k), hs = _trees(n_neurons, ncomp, seed=4)
    targets = configs.grad_targets(trees, seed=5)
    ht = [model.build(t.model(na, k, dt=DT), exact=True) for t in targets]
    rows = [[h.ncompts - 1] for h in hs]
    traces = _oracle_trace(oracle, ht, nsteps, rows)
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_FP64, wide_min=-1)
    b = eng.batch
    L, dchip, drav, dvm = eng.loss_gradient(nsteps, np.arange(n_neurons), np.array([r[0] for r in rows]),
                                            np.concatenate(traces, axis=1), K)
    eng.close()
    # 64 sampled (neuron, parameter) pairs, each under the per-sample rule
    rng = np.random.default_rng(5)
    npar = 3 * ncomp + 2
    picks = [(int(rng.integers(n_neurons)), int(rng.integers(npar))) for _ in range(64)]
    res = []
    for i, j in picks:
        t, h = trees[i], hs[i]
        g = configs.param_gradient(t, h, dchip[b.chip_start[i]:b.chip_start[i + 1]],
                                   drav[b.ravals_start[i]:b.ravals_start[i + 1]], na.Ek, dt=DT)
        res.append(fd_rule(oracle, t, (na, k), j, g[j], nsteps, rows[i], traces[i]))
    errs = np.array([r[1] for r in res])
    kinds = [r[0] for r in res]
    print("config-4 shape: loss %.6g; |rel err| vs FD(h=1e-6): median %.3g, 90%% %.3g, max %.3g; kinds %s"
          % (L, np.median(errs), np.quantile(errs, 0.9), errs.max(),
             {kk: kinds.count(kk) for kk in sorted(set(kinds))}))
    bad = [(picks[q], res[q]) for q in range(len(res)) if res[q][0] == "fail"]
    assert not bad, bad


@pytest.mark.gpu
def test_config4_full_size_vs_fd(oracle, gpu_engine):
    """Config 4 as configured: 4,096 trees x 64 compartments, 10,000 steps,
    checkpoints every 100, targets from gbar x U(0.8, 1.2). Target traces come
    from the FP64 engine (bit-identical to the oracle); 64 sampled physical
    parameters meet the per-sample rule against the oracle's losses."""
    n_neurons, ncomp, nsteps, K = 4096, 64, 10000, 100
    trees, (na, k), hs = _trees(n_neurons, ncomp, seed=4)
    targets = configs.grad_targets(trees, seed=5)
    ht = [model.build(t.model(na, k, dt=DT), exact=True) for t in targets]
    soma = np.array([h.ncompts - 1 for h in hs], dtype=np.int32)
    solver = np.arange(n_neurons, dtype=np.int32)
    et = gpu_engine.Engine(ht, precision=gpu_engine.PREC_FP64, wide_min=-1)
    et.register_outputs(solver, soma)
    tr = np.empty((nsteps, n_neurons))
    for n in range(nsteps):
        et.run(1)
        et.get_outputs_async(tr[n])
    et.close()
    eng = gpu_engine.Engine(hs, precision=gpu_engine.PREC_FP64, wide_min=-1)
    b = eng.batch
    L, dchip, drav, dvm = eng.loss_gradient(nsteps, solver, soma, tr, K)
    eng.close()
    rng = np.random.default_rng(5)
    npar = 3 * ncomp + 2
    picks = [(int(rng.integers(n_neurons)), int(rng.integers(npar))) for _ in range(64)]
    res = []
    for i, j in picks:
        g = configs.param_gradient(trees[i], hs[i], dchip[b.chip_start[i]:b.chip_start[i + 1]],
                                   drav[b.ravals_start[i]:b.ravals_start[i + 1]], na.Ek, dt=DT)
        res.append(fd_rule(oracle, trees[i], (na, k), j, g[j], nsteps, [soma[i]], tr[:, i:i + 1]))
    errs = np.array([r[1] for r in res])
    kinds = [r[0] for r in res]
    print("config 4 (4,096 trees): loss %.6g; |rel err| median %.3g, max %.3g; kinds %s"
          % (L, np.median(errs), errs.max(), {kk: kinds.count(kk) for kk in sorted(set(kinds))}))
    bad = [(picks[q], res[q]) for q in range(len(res)) if res[q][0] == "fail"]
    assert not bad, bad
