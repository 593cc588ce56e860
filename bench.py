#!/usr/bin/env python3
"""Benchmark of the GB300 hsolve step engine (one JSON line on rank 0).

Workload: 100,000 identical neurons x 16 compartments (1.6 M compartments),
config-0 morphology (soma 30x30 um + 15 dendrites 20x2 um) with somatic HH
Na/K and a dendritic K tabchannel at 36 S/m^2, seeded per-neuron inject
U(0.1, 0.5) nA, dt = 20 us, backward Euler. One step = one hsolve PROCESS
step over all compartments (channel program, elimination, Vm update).

  value    compartment-steps/s of the mixed-precision form, device-timed
           (CUDA events around the launches, inputs resident in HBM; the
           1.6 M-compartment state is larger than L2)
  forms    the same for the plain FP64 form, plus the mixed form's max|dVm|
           against the FP64 CPU oracle over 10,000 steps of a neuron sample
  e2e      the same metric through the C ABI with host buffers: every step
           copies the per-neuron inject currents host->device (h_in_msgs) and
           the somatic Vm of every neuron device->host (h_out_msgs), through
           gbh_run_io (the whole run's inputs and outputs in pinned host
           arrays, copied in blocks of IO_BLOCK steps on their own streams
           while neighbouring blocks step); `e2e.per_step_call` is the same
           I/O with one gbh_step_io call per step, `e2e.serial` the same I/O
           on one stream
  roofline HBM roofline of the step kernel (algorithmic bytes per
           compartment-step x compartment-steps per launch / launch time)

``--impl reference`` times the reference's own CPU step code (compiled from
its sources into oracle/_ref; the oracle's restatement where they are not
available) on every host core over a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "genesis-2.4_gb300"))

import numpy as np  # noqa: E402

N_NEURONS = 100_000
NCOMP = 16
GK_DEND = 36.0
DT = 20e-6
SEED = 3
IO_BLOCK = 16       # steps per host<->device transfer block of the end-to-end run
# algorithmic bytes per compartment-step for this workload (one streaming
# pass over per-compartment state and coefficients, tables on chip):
# FP64 (16+32)*16 + 28*15 + 17*16 + 18*16 = 1748 B per neuron; mixed 1469 B
ALG_BYTES = {"fp64": 1748.0 / NCOMP, "mixed": 1469.0 / NCOMP}
# random trees (8-256 compartments, Ca pools): algorithmic bytes per
# compartment-step, the per-compartment streaming pass of the mixed form
# (~76 B) plus the soma's channels and Ca pool spread over the mean tree
TREE_BYTES = 78.0
ACC_STEPS = 10_000
ACC_SAMPLE = 32
# differentiated form (gradient of a somatic-trace loss)
GRAD_NEURONS, GRAD_NCOMP, GRAD_STEPS, GRAD_K, GRAD_DT = 4096, 64, 10_000, 100, 25e-6


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return ws, rank, local, dist
    return 1, 0, 0, None


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", "gbh_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [l.strip().split(",") for l in open(self.path) if l.strip()]
            sm = [float(r[0]) for r in rows]
            mx = float(rows[0][1])
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            reasons = sorted({names[i] for r in rows for i in range(4) if r[2 + i].strip() == "Active"})
            return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": reasons,
                    "samples": len(sm)}
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def build_workload(n_neurons):
    from gbhsolve import configs
    t = time.time()
    hs, injects = configs.cables_replicated(n_neurons, NCOMP, seed=SEED, dt=DT, gk_dend=GK_DEND)
    log("workload built: %d neurons in %.1fs" % (n_neurons, time.time() - t))
    return hs, injects


def time_engine(eng, steps, warmup):
    eng.run(warmup)
    st0 = eng.stats()
    ms0, l0 = st0.device_ms, st0.launches
    eng.run(steps)
    st1 = eng.stats()
    return st1.device_ms - ms0, st1.launches - l0, st1


def _crossings(v, dt, thresh=0.0):
    """Upward threshold crossings of a trace, linearly interpolated (s)."""
    out = []
    for n in range(1, len(v)):
        if v[n - 1] < thresh <= v[n]:
            out.append((n - 1 + (thresh - v[n - 1]) / (v[n] - v[n - 1])) * dt)
    return out


def accuracy_sample(hs, precision, nsteps=ACC_STEPS, nsample=ACC_SAMPLE):
    """max|dVm| of the engine against the FP64 oracle over nsteps steps on a
    sample of neurons, and the deviation of somatic spike times (upward 0 V
    crossings, interpolated between steps)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    from gbhsolve import engine
    idx = np.linspace(0, len(hs) - 1, nsample).astype(int)
    sample = [hs[i] for i in idx]
    # the sample runs the kernels of the full workload: 32 neurons per warp
    # (a sample this small would otherwise go one neuron per warp)
    eng = engine.Engine(sample, precision=precision, wide_min=-1)
    orc = [pyoracle.Solver(h) for h in sample]
    soma = np.cumsum([h.ncompts for h in sample]) - 1      # the root is each solver's last row
    trace_e = np.empty((nsteps, len(sample)))
    trace_o = np.empty((nsteps, len(sample)))
    worst = 0.0
    for n in range(nsteps):
        eng.run(1)
        for s in orc:
            s.run(1)
        vm = eng.vm()
        ref = np.concatenate([s.vm for s in orc])
        worst = max(worst, float(np.max(np.abs(vm - ref))))
        trace_e[n] = vm[soma]
        trace_o[n] = ref[soma]
    eng.close()
    dt = float(sample[0].dt)
    dev, nspk, mismatch = 0.0, 0, 0
    for j in range(len(sample)):
        te, to = _crossings(trace_e[:, j], dt), _crossings(trace_o[:, j], dt)
        mismatch += abs(len(te) - len(to))
        for a, b in zip(te, to):
            dev = max(dev, abs(a - b))
            nspk += 1
    return worst, dev, nspk, mismatch


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def cpu_impl():
    """The CPU step code timed: the reference's own (compiled from its
    sources into oracle/_ref where they are available), else the oracle's
    restatement of it (bit-equal to it)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    pyoracle.ensure_built(with_reference=True)
    if os.path.exists(pyoracle.LIB_REF):
        return "reference", "reference"
    return "oracle", "port"


def cpu_sample_rate(hs, seconds=12.0):
    """The reference's step code (one core) compartment-steps/s over a
    bounded sample."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    impl, kind = cpu_impl()
    solvers = [pyoracle.Solver(h) for h in hs[:256]]
    steps = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for s in solvers:
            s.run(20, impl)
        steps += 20
    el = time.perf_counter() - t0
    cs = steps * len(solvers) * NCOMP
    return cs / el, kind, "%d neurons x %d compartments x %d steps (%.1f s)" % (len(solvers), NCOMP, steps, el)


def _cpu_worker(args):
    n, steps, seed, impl = args
    sys.path.insert(0, os.path.join(REPO, "genesis-2.4_gb300"))
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    from gbhsolve import configs
    hs, _ = configs.cables_replicated(n, NCOMP, seed=seed, dt=DT, gk_dend=GK_DEND)
    solvers = [pyoracle.Solver(h) for h in hs]
    t0 = time.perf_counter()
    for s in solvers:
        s.run(steps, impl)
    return n * NCOMP * steps, time.perf_counter() - t0


def adjoint_measure(device, n_neurons=GRAD_NEURONS, nsteps=GRAD_STEPS):
    """Gradient workload: 4,096 seeded random binary trees x 64 compartments
    with Na, K and leak on every compartment, dt 25 us, backward Euler; loss =
    summed squared somatic Vm error over 10,000 steps against traces of the
    same trees with every gbar scaled by U(0.8, 1.2). Times gbh_loss_gradient
    against the plain FP64 forward (gbh_run) of the same steps on the same
    engine: every step's state kept in device memory (~84 GB), and with
    checkpoints every 100 steps (each segment recomputed), which must give
    the same bits."""
    import torch
    from gbhsolve import configs, engine, model
    t0 = time.time()
    trees, (na, k) = configs.grad_trees(n_neurons, ncomp=GRAD_NCOMP, seed=4)
    targets = configs.grad_targets(trees, seed=5)
    hs = [model.build(t.model(na, k, dt=GRAD_DT), exact=True) for t in trees]
    ht = [model.build(t.model(na, k, dt=GRAD_DT), exact=True) for t in targets]
    solver = np.arange(n_neurons, dtype=np.int32)
    soma = np.array([h.ncompts - 1 for h in hs], dtype=np.int32)
    log("gradient workload built in %.1f s" % (time.time() - t0))
    # target traces from the FP64 engine (bit-identical to the CPU oracle)
    et = engine.Engine(ht, precision=engine.PREC_FP64, device=device)
    et.register_outputs(solver, soma)
    trace = torch.empty((nsteps, n_neurons), dtype=torch.float64, pin_memory=True)
    tr = trace.numpy()
    stream = torch.cuda.Stream()
    for n in range(nsteps):
        et.run_async(1, stream.cuda_stream)
        et.get_outputs_async(tr[n], stream.cuda_stream)
    stream.synchronize()
    et.close()
    eng = engine.Engine(hs, precision=engine.PREC_FP64, device=device, wide_min=-1)   # the adjoint runs lane-mapped
    st0 = eng.get_state()
    ms0 = eng.stats().device_ms
    eng.run(nsteps)
    fwd_ms = eng.stats().device_ms - ms0
    eng.set_state(vm=st0["vm"], chip=st0["chip"])
    # every step's state kept in device memory (checkpoint_every 0), then
    # checkpoints every GRAD_K steps with each segment recomputed: same bits
    launches0 = eng.stats().launches
    t1 = time.time()
    loss, dchip, drav, dvm = eng.loss_gradient(nsteps, solver, soma, tr, 0)
    wall = time.time() - t1
    st = eng.stats()
    grad_ms = st.grad_forward_ms + st.grad_reverse_ms
    kept = int(st.grad_kept_steps)
    launches = int(st.launches - launches0)
    loss_c, dchip_c, drav_c, dvm_c = eng.loss_gradient(nsteps, solver, soma, tr, GRAD_K)
    stc = eng.stats()
    grad_c_ms = stc.grad_forward_ms + stc.grad_reverse_ms
    same = bool(loss_c == loss and np.array_equal(dchip_c, dchip) and np.array_equal(drav_c, drav)
                and np.array_equal(dvm_c, dvm))
    eng.close()
    finite = bool(np.all(np.isfinite(dchip)) and np.all(np.isfinite(drav)) and np.all(np.isfinite(dvm)))
    log("gradient: forward %.1f ms, gradient %.1f ms (forward pass %.1f, reverse %.1f, every step kept: %d), "
        "ratio %.2f; checkpointed every %d: %.1f ms (ratio %.2f), same bits %s; loss %.6g"
        % (fwd_ms, grad_ms, st.grad_forward_ms, st.grad_reverse_ms, kept, grad_ms / fwd_ms, GRAD_K, grad_c_ms,
           grad_c_ms / fwd_ms, same, loss))
    return {"workload": "grad-trees-%dx%d: %d random binary trees x %d compartments, Na/K/leak on every "
                        "compartment, dt 25 us, backward Euler, somatic-trace loss" % (n_neurons, GRAD_NCOMP, n_neurons, GRAD_NCOMP),
            "steps": nsteps, "checkpoint_every": 0, "every_step_kept": kept, "dtype": "f64",
            "forward_ms": fwd_ms, "gradient_ms": grad_ms, "forward_pass_ms": st.grad_forward_ms,
            "reverse_pass_ms": st.grad_reverse_ms, "gradient_wall_s": wall,
            "ratio_gradient_over_forward": grad_ms / fwd_ms,
            "ratio_backward_over_forward": st.grad_reverse_ms / fwd_ms, "loss": loss, "gradients_finite": finite,
            "launches": launches,
            "checkpointed": {"checkpoint_every": GRAD_K, "gradient_ms": grad_c_ms,
                             "checkpoint_pass_ms": stc.grad_forward_ms, "reverse_pass_ms": stc.grad_reverse_ms,
                             "ratio_gradient_over_forward": grad_c_ms / fwd_ms,
                             "same_bits_as_every_step_kept": same}}


def other_configs(device, n_trees=50_000):
    """Throughput of the other workloads (parity-test cases; not the headline):
    cables-1k-x16 (1,000 x 16-compartment cables, FP64, 200 steps), the
    4,000-cell spiking network (2 % connectivity, dt 0.1 ms, FP64, seeded
    tonic drive U(0.05, 0.3) nA so that it spikes) with and without
    CUDA-graph replay, and random trees 8-256 compartments with Ca
    pools (50,000 neurons, 3.6 M compartments, FP64 and mixed, graph replay,
    500 steps)."""
    from gbhsolve import configs, engine, model
    out = {}

    def rate(eng, steps, warm):
        eng.run(warm)
        ms0 = eng.stats().device_ms
        eng.run(steps)
        return eng.stats().device_ms - ms0

    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle

    hs0 = [model.build(m) for m in configs.cables(1000, per_neuron_solvers=True)]
    eng = engine.Engine(hs0, precision=engine.PREC_FP64, device=device)
    ms = rate(eng, 200, 20)
    out["cables-1k-x16"] = {"compartments": 16_000, "steps": 200, "ms": ms, "value": 16_000 * 200 / (ms / 1e3),
                            "dtype": "f64"}
    eng.close()
    # the mixed form against the reference's FP64 step (the oracle) over the
    # configured 200 steps, every neuron
    ref = []
    for h in hs0:
        o = pyoracle.Solver(h)
        o.run(200)
        ref.append(o.vm.copy())
    mx = engine.Engine(hs0, precision=engine.PREC_MIXED, device=device)
    mx.run(200)
    out["cables-1k-x16"]["mixed_max_abs_dvm_vs_fp64_oracle_V"] = float(
        max(np.max(np.abs(a - b)) for a, b in zip(mx.get_state()["vm"], ref)))
    mx.close()

    ms1, syn = configs.hh_network(4000)
    drive = np.random.default_rng(1).uniform(0.05e-9, 0.3e-9, size=len(ms1))   # tonic drive, recorded choice
    for m, x in zip(ms1, drive):
        m.compartments[0].inject = float(x)
    hs1 = [model.build(m) for m in ms1]
    esyn, _ = configs.network_synapses(hs1, syn)
    net = {"cells": 4000, "synapses": int(len(esyn["target_solver"])), "steps": 5000, "dtype": "f64",
           "drive": "inject U(0.05, 0.3) nA, seed 1"}
    fp64_counts = fp64_vm = None
    for graph in (False, True):
        eng = engine.Engine(hs1, synapses=esyn, precision=engine.PREC_FP64, device=device, use_graph=graph)
        st = eng.stats()
        if graph:
            # a graph is captured per step count: the untimed first 5,000-step
            # run captures the one the timed run replays; its spike counts
            # after the same 5,100 steps must equal the per-launch engine's
            eng.run(100)
            eng.run(5000)
            same = bool(np.array_equal(eng.spike_counts(), fp64_counts))
            ms0 = eng.stats().device_ms
            eng.run(5000)
            ms = eng.stats().device_ms - ms0
        else:
            ms = rate(eng, 5000, 100)
        key = "graph" if graph else "launches"
        net[key] = {"ms": ms, "steps_per_s": 5000 / (ms / 1e3), "value": 4000 * 5000 / (ms / 1e3),
                    "spikes": int(eng.spike_counts().sum()), "cooperative": int(st.cooperative),
                    "specialised_kernels": int(st.jit_kernels)}
        if graph:
            net[key].update({"timed": "replay of the captured 5,000-step graph (steps 5,100-10,100)",
                             "spike_counts_equal_launches_at_5100": same})
        else:
            fp64_counts, fp64_vm = eng.spike_counts(), eng.vm()
        eng.close()
    # the mixed form over the same 5,100 steps against the FP64 engine (which
    # equals the reference's step code bit for bit): spike counts per cell
    mx = engine.Engine(hs1, synapses=esyn, precision=engine.PREC_MIXED, device=device)
    mx.run(5100)
    mc = mx.spike_counts()
    net["mixed"] = {"spike_count_mismatch_cells": int(np.sum(mc != fp64_counts)), "spikes": int(mc.sum()),
                    "max_abs_dvm_vs_fp64_V": float(np.max(np.abs(mx.vm() - fp64_vm))), "steps": 5100}
    mx.close()
    out["hh-network-4000"] = net

    # SETUP of the 50,000 hsolves (the restated h_hh_chip_init / do_hget_children
    # / h_funcs_init, with the model generation) on every host core
    ts = time.perf_counter()
    hs2 = model.build_generated(configs.random_trees, n_trees, seed=2)
    setup_s = time.perf_counter() - ts
    M2 = sum(h.ncompts for h in hs2)
    trees = {"neurons": n_trees, "compartments": M2, "steps": 500,
             "timed": "500 of the configured 5,000 steps (a rate; neurons are independent)",
             "hsolve_setup_s": setup_s, "hsolve_setup_processes": model.setup_workers()}
    for form, prec in (("fp64", engine.PREC_FP64), ("mixed", engine.PREC_MIXED)):
        tc = time.perf_counter()
        eng = engine.Engine(hs2, precision=prec, device=device, use_graph=True)
        setup = time.perf_counter() - tc
        st = eng.stats()
        ms = rate(eng, 500, 20)
        trees[form] = {"ms": ms, "value": M2 * 500 / (ms / 1e3), "tiles": int(st.tiles),
                       "wide_tiles": int(st.wide_tiles), "stack_tiles": int(st.stack_tiles),
                       "specialised_kernels": int(st.jit_kernels), "steps_per_launch": int(st.steps_per_launch),
                       "engine_setup_s": setup,
                       "hbm_frac": TREE_BYTES * M2 * 500 / (ms / 1e3) / 1e9 / peaks()[0]}
        eng.close()
    # the mixed form against the reference's FP64 step over the configured
    # 5,000 steps on a seeded 1-in-500 sample of the trees
    sample = hs2[::500]
    acc, dev, nspk, mism = accuracy_sample(sample, engine.PREC_MIXED, nsteps=5000, nsample=len(sample))
    trees["mixed"].update({"max_abs_dvm_vs_fp64_oracle_V": acc, "spike_time_max_dev_s": dev, "spikes_compared": nspk,
                           "spike_count_mismatches": mism, "accuracy_sample_neurons": len(sample),
                           "accuracy_steps": 5000})
    out["random-trees-ca"] = trees
    log("other configs: %s" % json.dumps(out))
    return out


def run_reference(args, ws, rank, dist):
    """The reference's CPU step code on every host core."""
    if rank != 0:
        return 0
    import multiprocessing as mp
    impl, kind = cpu_impl()
    cores = os.cpu_count() or 1
    per = 96                       # neurons per worker per step batch
    nst = 100                      # steps per neuron per timed sample (amortises the per-call overhead)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_cpu_worker, [(8, 5, k, impl) for k in range(cores)])   # warm the workers
        vals = []
        for _ in range(args.warmup):
            pool.map(_cpu_worker, [(per, nst, k, impl) for k in range(cores)])
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_cpu_worker, [(per, nst, k, impl) for k in range(cores)])
            wall = time.perf_counter() - t0
            cs = sum(r[0] for r in res)
            # each worker's in-process time; the slowest one sets the step
            # (pool dispatch, the workers' model build excluded)
            vals.append(cs / max(max(r[1] for r in res), 1e-9))
    value = float(np.median(vals))
    line = {
        "metric": "compartment-steps/s", "value": value, "unit": "compartment-steps/s",
        "impl": "reference", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "cables-100k-x16 (config 3 morphology, dendritic K)", "sample_neurons":
                   per * cores, "steps_per_sample": nst},
        "cpu_baseline": {"value": value, "unit": "compartment-steps/s", "cores": cores, "kind": kind,
                         "cpu": cpu_model(),
                         "code": "the reference's own step code (hines_4chip.c, hines_solve.c, ...) compiled "
                                 "with its -O2" if kind == "reference" else "the oracle's restatement",
                         "sample": "%d workers x %d neurons x 16 compartments x %d steps per timed step; value: "
                                   "compartment-steps over the slowest worker's in-process time"
                                   % (cores, per, nst)},
        "e2e": {"value": value, "unit": "compartment-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "reference_cuda_backend": reference_cuda_backend(),
    }
    print(json.dumps(line), flush=True)
    return 0


def reference_cuda_backend():
    """The reference's own GPU arm on the cables workload of 1,000 x 16
    compartments (oracle/ref_cuda.py, its own process); beside the CPU arm,
    not the headline."""
    try:
        r = subprocess.run([sys.executable, os.path.join(REPO, "oracle", "ref_cuda.py")], capture_output=True,
                           text=True, timeout=900)
        lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
        if not lines:
            return {"unavailable": "no result (exit %d): %s" % (r.returncode, r.stderr.strip()[-300:])}
        return json.loads(lines[-1])
    except Exception as ex:  # noqa: BLE001 -- recorded in the line, never fatal to the arm
        return {"unavailable": "%s: %s" % (type(ex).__name__, ex)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--neurons", type=int, default=N_NEURONS)
    ap.add_argument("--steps-per-launch", type=int, default=0)
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-adjoint", action="store_true")
    ap.add_argument("--skip-configs", action="store_true")
    ap.add_argument("--profile-form", choices=["fp64", "mixed"],
                    help="time only this form's step loop (for profiler launch lists and captures)")
    ap.add_argument("--profile-adjoint", type=int, nargs=2, metavar=("NEURONS", "STEPS"),
                    help="run only the gradient workload at this size")
    ap.add_argument("--wide-min", type=int, default=0,
                    help="--profile-trees: the engine's wide_min (0 mapping chosen by trial, < 0 never wide)")
    ap.add_argument("--no-jit", action="store_true",
                    help="--profile-trees / --profile-network: interpret every program (no specialised kernels)")
    ap.add_argument("--profile-network", type=int, metavar="STEPS",
                    help="run only the 4,000-cell network (FP64, tonic drive) for this many steps")
    ap.add_argument("--profile-trees", type=int, metavar="NEURONS",
                    help="run only random trees (8-256 compartments, Ca) of this many neurons, the form of "
                         "--profile-form (default mixed), steps_per_launch --steps-per-launch (default 64); "
                         "the timed steps run between cudaProfilerStart/Stop")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local, dist = dist_setup()
    if args.impl == "reference":
        return run_reference(args, ws, rank, dist)

    import torch
    torch.cuda.set_device(local)
    from gbhsolve import engine

    if args.profile_adjoint:
        print(json.dumps(adjoint_measure(local, *args.profile_adjoint)), flush=True)
        return 0
    if args.profile_trees:
        from gbhsolve import configs, model
        ht = model.build_generated(configs.random_trees, args.profile_trees, seed=2)
        prec = engine.PREC_FP64 if args.profile_form == "fp64" else engine.PREC_MIXED
        eng = engine.Engine(ht, precision=prec, steps_per_launch=args.steps_per_launch or 64, device=local,
                            wide_min=args.wide_min, jit=not args.no_jit)
        eng.run(args.warmup)
        eng.vm()
        ms0 = eng.stats().device_ms
        torch.cuda.profiler.start()
        eng.run(args.steps)
        eng.vm()
        torch.cuda.profiler.stop()
        st = eng.stats()
        us = (st.device_ms - ms0) / args.steps * 1e3
        ncs = sum(h.ncompts for h in ht)
        log("random trees %d (%s): %.1f us/step on the device (%.3g compartment-steps/s), %d tiles "
            "(%d wide, %d stack), %d steps per launch" % (args.profile_trees, args.profile_form, us,
                                                          ncs / (us * 1e-6), st.tiles, st.wide_tiles,
                                                          st.stack_tiles, st.steps_per_launch))
        eng.close()
        return 0
    if args.profile_network:
        from gbhsolve import configs, model
        ms1, syn = configs.hh_network(4000)
        drive = np.random.default_rng(1).uniform(0.05e-9, 0.3e-9, size=len(ms1))
        for m, x in zip(ms1, drive):
            m.compartments[0].inject = float(x)
        hs1 = [model.build(m) for m in ms1]
        esyn, _ = configs.network_synapses(hs1, syn)
        eng = engine.Engine(hs1, synapses=esyn, precision=engine.PREC_FP64, device=local, jit=not args.no_jit)
        eng.run(args.warmup)
        ms0 = eng.stats().device_ms
        eng.run(args.profile_network)
        ms = eng.stats().device_ms - ms0
        log("network 4000: %.2f us/step, %d spikes" % (ms / args.profile_network * 1e3, eng.spike_counts().sum()))
        eng.close()
        return 0
    hs, injects = build_workload(args.neurons)
    if args.profile_form:
        prec = engine.PREC_MIXED if args.profile_form == "mixed" else engine.PREC_FP64
        eng = engine.Engine(hs, precision=prec, steps_per_launch=args.steps_per_launch, device=local)
        ms, launches, st = time_engine(eng, args.steps, args.warmup)
        log("%s: %.3f ms for %d steps, %d launches, %d steps/launch" % (args.profile_form, ms, args.steps, launches,
                                                                    st.steps_per_launch))
        eng.close()
        return 0
    M = args.neurons * NCOMP
    results = {}
    for form, prec in (("fp64", engine.PREC_FP64), ("mixed", engine.PREC_MIXED)):
        # engine setup: descriptor packing, decode (threaded over solvers),
        # layout, upload, specialisation (NVRTC) and autotuning
        tc = time.perf_counter()
        eng = engine.Engine(hs, precision=prec, steps_per_launch=args.steps_per_launch, device=local)
        setup_s = time.perf_counter() - tc
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        with Clocks(local) as clk:
            ms, launches, st = time_engine(eng, args.steps, args.warmup)
        torch.cuda.synchronize()
        if dist:
            t = torch.tensor([ms], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        results[form] = dict(ms=ms, launches=launches, spl=st.steps_per_launch,
                             value=M * ws * args.steps / (ms / 1e3), clocks=clk.summary(), eng=eng,
                             setup_s=setup_s)
        log("%s: %.3f ms for %d steps, %d launches, %d specialised kernels (min blocks %d, %s form),"
            " %d steps/launch -> %.3e cs/s (engine setup %.2f s)"
            % (form, ms, args.steps, launches, st.jit_kernels, st.jit_min_blocks,
               ["unrolled", "compact", "unrolled/shared-rows"][st.jit_compact], st.steps_per_launch,
               results[form]["value"], setup_s))
        if form == "fp64":
            eng.close()

    # end to end through the C ABI with host buffers (mixed form): every step
    # copies the inject currents host->device and the somatic Vm of every
    # neuron device->host. `e2e`: gbh_step_io (copies on their own stream,
    # overlapping the neighbouring steps); `e2e_serial`: the same I/O with
    # set_inputs_async / run_async / get_outputs_async on one stream.
    eng = results["mixed"]["eng"]
    nh = len(hs)
    eng.register_inputs(np.arange(nh, dtype=np.int32),
                        np.full(nh, int(hs[0].compchips[NCOMP - 1]) + 1, dtype=np.int64))
    eng.register_outputs(np.arange(nh, dtype=np.int32), np.full(nh, NCOMP - 1, dtype=np.int32))
    inj = np.array([float(np.float32(x)) for x in injects])
    pin_in = [torch.empty(nh, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    pin_out = [torch.empty(nh, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    for x in pin_in:
        x[:] = inj
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream

    def timed(loop):
        for k in range(args.warmup):
            loop(k)
        eng.io_sync()
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if dist:
            dist.barrier()
        e0.record(stream)
        for k in range(args.steps):
            loop(k)
        eng.io_sync()
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1)
        if dist:
            t = torch.tensor([ms], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    def piped(k):
        eng.step_io(pin_in[k % 3], pin_out[k % 3], 1, sh)

    def serial(k):
        eng.set_inputs_async(pin_in[0], sh)
        eng.run_async(1, sh)
        eng.get_outputs_async(pin_out[0], sh)

    # gbh_run_io: the whole run's per-step inputs and outputs in host arrays
    # (steps x neurons, pinned), streamed in blocks of IO_BLOCK steps
    run_in = torch.empty((max(args.steps, args.warmup), nh), dtype=torch.float64, pin_memory=True).numpy()
    run_out = torch.empty((max(args.steps, args.warmup), nh), dtype=torch.float64, pin_memory=True).numpy()
    run_in[:] = inj

    def streamed_run():
        eng.run_io(run_in[:args.warmup], run_out[:args.warmup], args.warmup, IO_BLOCK, sh)
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if dist:
            dist.barrier()
        e0.record(stream)
        eng.run_io(run_in[:args.steps], run_out[:args.steps], args.steps, IO_BLOCK, sh)
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1)
        if dist:
            t = torch.tensor([ms], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    e2e_ms = streamed_run()
    e2e_call_ms = timed(piped)
    e2e_serial_ms = timed(serial)
    e2e_val = M * ws * args.steps / (e2e_ms / 1e3)
    e2e_call = M * ws * args.steps / (e2e_call_ms / 1e3)
    e2e_serial = M * ws * args.steps / (e2e_serial_ms / 1e3)
    log("e2e: %.3e cs/s block-streamed (gbh_run_io), %.3e one call per step (gbh_step_io), %.3e serial"
        % (e2e_val, e2e_call, e2e_serial))
    eng.close()

    # accuracy of the mixed form against the FP64 oracle
    acc = spk_dev = None
    nspk = spk_mismatch = None
    if rank == 0 and not args.skip_accuracy:
        acc, spk_dev, nspk, spk_mismatch = accuracy_sample(hs, engine.PREC_MIXED)
        log("mixed max|dVm| over %d steps: %.3e V; spike times: %d spikes, max deviation %.3e s, count "
            "mismatches %d" % (ACC_STEPS, acc, nspk, spk_dev, spk_mismatch))

    adj = None
    if rank == 0 and not args.skip_adjoint:
        adj = adjoint_measure(local)
    other = None
    if rank == 0 and not args.skip_configs:
        other = other_configs(local)

    cpu = None
    if rank == 0 and not args.skip_cpu:
        v, kind, sample = cpu_sample_rate(hs)
        cpu = {"value": v, "unit": "compartment-steps/s", "cores": 1, "kind": kind, "cpu": cpu_model(),
               "sample": sample}

    peak, peak_kind = peaks()
    r = results["mixed"]
    launch_ms = r["ms"] / max(r["launches"], 1)
    units = M * args.steps / max(r["launches"], 1)     # compartment-steps one launch processes
    achieved = ALG_BYTES["mixed"] * units / (launch_ms / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(REPO, "profiles", "k_steps_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        if "bytes_per_compartment_step_mixed" in tj:
            traffic = tj["bytes_per_compartment_step_mixed"] * units
    if rank == 0:
        line = {
            "metric": "compartment-steps/s", "value": r["value"], "unit": "compartment-steps/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-gates/f64-elimination", "data": "synthetic",
            "config": {"workload": "cables-100k-x16: 100,000 neurons x 16 compartments, somatic HH Na/K, "
                                   "dendritic K 36 S/m^2, dt 20 us, backward Euler",
                       "compartments": M, "form": "batched mixed precision",
                       "steps_per_launch": r["spl"], "autotuned": args.steps_per_launch == 0,
                       "l2": "state 1.6M compartments > L2, no flush"},
            "forms": {"fp64": {"value": results["fp64"]["value"], "ms_per_step": results["fp64"]["ms"] / args.steps,
                               "dtype": "f64", "engine_setup_s": results["fp64"]["setup_s"]},
                      "mixed": {"value": r["value"], "ms_per_step": r["ms"] / args.steps,
                                "engine_setup_s": r["setup_s"],
                                "max_abs_dvm_vs_fp64_oracle_V": acc, "accuracy_steps": ACC_STEPS,
                                "spike_time_max_dev_s": spk_dev, "spikes_compared": nspk,
                                "spike_count_mismatches": spk_mismatch,
                                "accuracy_sample_neurons": ACC_SAMPLE}},
            "speedup_mixed_over_fp64": r["value"] / results["fp64"]["value"],
            "e2e": {"value": e2e_val, "unit": "compartment-steps/s", "h2d_bytes_per_step": nh * 8,
                    "d2h_bytes_per_step": nh * 8,
                    "api": "gbh_run_io (per-step inputs/outputs of the whole run, host<->device copies "
                           "streamed in blocks of %d steps overlapping the steps)" % IO_BLOCK,
                    "per_step_call": {"value": e2e_call, "api": "gbh_step_io, one call per step, copies pipelined"},
                    "serial": {"value": e2e_serial, "api": "set_inputs_async + run_async + get_outputs_async"}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "gbh_jit (specialised mixed step)", "launch_ms": launch_ms,
                         "alg_bytes_per_compartment_step": ALG_BYTES["mixed"]},
            "cpu_baseline": cpu,
            "adjoint": adj,
            "other_configs": other,
            "gpu_launches": int(r["launches"]),
            "clocks": r["clocks"],
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
