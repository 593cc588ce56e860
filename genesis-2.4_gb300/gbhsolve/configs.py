"""Model definitions: the reference's golden model and the five benchmark
workloads, as seeded synthetic models (no datasets are involved).

Parameter values that a GENESIS script would pass through an SLI expression
are rounded with :func:`sli` first, element fields with float storage are
rounded by the builder.
"""
from __future__ import annotations

import math

import numpy as np

from .model import (BEULER, CRANK, CaConcen, ChannelType, Compartment, GateTables, Model,
                    SpikeGen, SynChan, TabChannel, f32, setup_alpha, setup_tau_table, sli)

PI = 3.141592653589793


def hh_channels(erest: float, xdivs=3000, xmin=-0.1, xmax=0.05):
    """Hodgkin-Huxley Na and K tabchannels as set up by ``setupalpha`` in
    genesis/Scripts/benchmark/hh1952_ap_verify.g:45-63 for resting potential
    ``erest``. Returns (Na, K) channel types."""
    ena = erest + 0.115
    ek = erest - 0.012
    na_x = [sli(100000.0 * (0.025 + erest)), -100000.0, -1.0, sli(-1.0 * (0.025 + erest)), -0.01,
            4000.0, 0.0, 0.0, sli(0.0 - erest), 0.018]
    na_y = [70.0, 0.0, 0.0, sli(0.0 - erest), 0.02,
            1000.0, 0.0, 1.0, sli(-0.03 - erest), -0.01]
    k_x = [sli(10000.0 * (0.010 + erest)), -10000.0, -1.0, sli(-1.0 * (0.010 + erest)), -0.01,
           125.0, 0.0, 0.0, sli(0.0 - erest), 0.08]
    na = ChannelType("Na_chan", Ek=sli(ena), Xpower=3, Ypower=1,
                     X=GateTables(*setup_alpha(na_x, xdivs, xmin, xmax)),
                     Y=GateTables(*setup_alpha(na_y, xdivs, xmin, xmax)))
    k = ChannelType("K_chan", Ek=sli(ek), Xpower=4,
                    X=GateTables(*setup_alpha(k_x, xdivs, xmin, xmax)))
    return na, k


# --------------------------------------------------------------------------
# hh1952_ap_verify.g: the reference's chanmode-4 CPU known-answer model
# (cluster_bringup/accel_regression_golden.txt:4 ap_cpu RESULT_VM)
# --------------------------------------------------------------------------
def ap_verify(n_neurons: int = 8, inject: float = 2e-9) -> Model:
    erest = -0.070
    soma_l = soma_d = 20e-6
    area = soma_l * PI * soma_d
    xarea = PI * (soma_d / 2) * (soma_d / 2)
    na, k = hh_channels(erest)
    comps = []
    for _ in range(n_neurons):
        c = Compartment(Em=sli(erest + 0.010613), Rm=sli(0.333333 / area), Cm=sli(0.01 * area),
                        Ra=sli(0.3 * soma_l / xarea), initVm=sli(erest), inject=sli(inject))
        c.children = [TabChannel(na, Gbar=sli(1200.0 * area)), TabChannel(k, Gbar=sli(360.0 * area))]
        comps.append(c)
    return Model(comps, dt=sli(10e-6), method=BEULER)


AP_VERIFY_GOLDEN = "-0.02143485882"   # 8 neurons, 10 + 200 steps, cell0 Vm


# --------------------------------------------------------------------------
# Cable neurons (configs 0 and 3)
# --------------------------------------------------------------------------
def cable_neuron(na, k, inject, ncomp=16, erest=-0.065, soma=(30e-6, 30e-6), dend=(20e-6, 2e-6),
                 rm=0.33, cm=0.01, ra=0.3, gna=1200.0, gk=360.0, gk_dend=0.0, base=0):
    """One unbranched cable: soma root plus ``ncomp-1`` dendrites in a chain.
    Returns the compartments, parents indexed from ``base``."""
    sl, sd = soma
    dl, dd = dend
    sa, sx = sl * PI * sd, PI * (sd / 2) ** 2
    da, dx = dl * PI * dd, PI * (dd / 2) ** 2
    out = []
    s = Compartment(Em=sli(erest), Rm=sli(rm / sa), Cm=sli(cm * sa), Ra=sli(ra * sl / sx),
                    initVm=sli(erest), inject=sli(inject), parent=-1)
    s.children = [TabChannel(na, Gbar=sli(gna * sa)), TabChannel(k, Gbar=sli(gk * sa))]
    out.append(s)
    for c in range(1, ncomp):
        d = Compartment(Em=sli(erest), Rm=sli(rm / da), Cm=sli(cm * da), Ra=sli(ra * dl / dx),
                        initVm=sli(erest), parent=base + c - 1)
        if gk_dend:
            d.children = [TabChannel(k, Gbar=sli(gk_dend * da))]
        out.append(d)
    return out


def cables(n_neurons: int, ncomp=16, seed=0, dt=20e-6, method=BEULER, gk_dend=0.0,
           inject_range=(0.1e-9, 0.5e-9), per_neuron_solvers=False, erest=-0.065):
    """Config 0 (gk_dend=0) / config 3 (gk_dend=36 S/m^2) cable populations.

    Returns a list of Models: one hsolve holding every neuron, or one hsolve
    per neuron when ``per_neuron_solvers``."""
    rng = np.random.default_rng(seed)
    injects = rng.uniform(inject_range[0], inject_range[1], size=n_neurons)
    na, k = hh_channels(erest)
    if per_neuron_solvers:
        return [Model(cable_neuron(na, k, float(injects[i]), ncomp, erest=erest, gk_dend=gk_dend),
                      dt=sli(dt), method=method) for i in range(n_neurons)]
    comps = []
    for i in range(n_neurons):
        comps += cable_neuron(na, k, float(injects[i]), ncomp, erest=erest, gk_dend=gk_dend,
                              base=len(comps))
    return [Model(comps, dt=sli(dt), method=method)]


# --------------------------------------------------------------------------
# Random trees (configs 2 and 4)
# --------------------------------------------------------------------------
def random_binary_tree(rng, ncomp):
    """Parents of a seeded random binary tree with ``ncomp`` nodes: every node
    gets zero or two children (a single chain link where one node is left)."""
    parents = [-1]
    frontier = [0]
    while len(parents) < ncomp:
        j = int(rng.integers(len(frontier)))
        p = frontier.pop(j)
        nkids = 2 if ncomp - len(parents) >= 2 else 1
        for _ in range(nkids):
            parents.append(p)
            frontier.append(len(parents) - 1)
    return parents


def ca_channels(erest=-0.065):
    """Ca channel (high-threshold, X^2) feeding the pool and a Ca-dependent K
    channel (Z gate on the conc axis, 3000 divs over 0..1 mM)."""
    eca = 0.128
    cax = [sli(1.6e3), 0.0, 1.0, sli(-0.005 - 0.060 - erest - 0.005), -0.0139,
           sli(20.0), 0.0, 1.0, sli(0.0 - erest - 0.065 + 0.0011 * 0 + 0.001), 0.005]
    ca = ChannelType("Ca_chan", Ek=eca, Xpower=2, X=GateTables(*setup_alpha(cax)))

    def kca_rates(c):
        cc = max(c, 1e-9)
        alpha = 500.0 * cc / (cc + 1.5e-4)   # per s, half activation at 0.15 mM
        beta = 40.0
        tau = 1.0 / (alpha + beta)
        return tau, alpha * tau

    kca = ChannelType("KCa_chan", Ek=erest - 0.012, Zpower=1, Z_conc=True,
                      Z=GateTables(*setup_tau_table(kca_rates, 3000, 0.0, 1.0)))
    return ca, kca


def random_tree_neuron(rng, ncomp, na, k, ca, kca, inject, erest=-0.065, dend_len=20e-6,
                       soma=(30e-6, 30e-6), rm=0.33, cm=0.01, ra=0.3, with_ca=True,
                       gna=1200.0, gk=360.0, dia_range=(0.5e-6, 3e-6)):
    parents = random_binary_tree(rng, ncomp)
    out = []
    sl, sd = soma
    sa, sx = sl * PI * sd, PI * (sd / 2) ** 2
    s = Compartment(Em=sli(erest), Rm=sli(rm / sa), Cm=sli(cm * sa), Ra=sli(ra * sl / sx),
                    initVm=sli(erest), inject=sli(inject), parent=-1)
    s.children = [TabChannel(na, Gbar=sli(gna * sa)), TabChannel(k, Gbar=sli(gk * sa))]
    if with_ca:
        shell_vol = sa * 0.1e-6           # 0.1 um sub-membrane shell
        B = 1.0 / (2 * 96485.3415 * shell_vol)
        s.children += [TabChannel(ca, Gbar=sli(40.0 * sa), flux_to=4),
                       TabChannel(kca, Gbar=sli(100.0 * sa), conc_src=4),
                       CaConcen(tau=0.02, B=B, Ca_base=5e-5, thick=0.1e-6)]
    out.append(s)
    # one draw per dendrite, in order (the same stream as scalar draws)
    dias = rng.uniform(dia_range[0], dia_range[1], size=ncomp - 1).tolist() if ncomp > 1 else []
    em = sli(erest)
    for c in range(1, ncomp):
        dd = dias[c - 1]
        da, dx = dend_len * PI * dd, PI * (dd / 2) ** 2
        out.append(Compartment(Em=em, Rm=sli(rm / da), Cm=sli(cm * da),
                               Ra=sli(ra * dend_len / dx), initVm=em, parent=parents[c]))
    return out


def random_trees(n_neurons, seed=2, size_range=(8, 256), dt=20e-6, with_ca=True,
                 inject_range=(0.0, 1e-9), method=BEULER, start=0, stop=None):
    """Config 2: one hsolve per neuron, log-uniform sizes. Sizes and injects
    are drawn for all ``n_neurons`` from ``seed``; neuron i's branching and
    diameters from its own generator seeded by (seed, i). So neurons
    [start, stop) can be generated alone (model.build_generated sets up
    the 50,000 on every core) and equal those of the whole set."""
    rng = np.random.default_rng(seed)
    na, k = hh_channels(-0.065)
    ca, kca = ca_channels()
    lo, hi = size_range
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi + 1), size=n_neurons)).astype(int)
    sizes = np.clip(sizes, lo, hi)
    injects = rng.uniform(inject_range[0], inject_range[1], size=n_neurons)
    models = []
    for i in range(start, n_neurons if stop is None else stop):
        comps = random_tree_neuron(np.random.default_rng((seed, i)), int(sizes[i]), na, k, ca, kca,
                                   float(injects[i]), with_ca=with_ca)
        models.append(Model(comps, dt=sli(dt), method=method))
    return models


# --------------------------------------------------------------------------
# Spiking network (config 1)
# --------------------------------------------------------------------------
def hh_network(n_cells=4000, frac_exc=0.8, p_conn=0.02, seed=1, dt=1e-4, delay=1e-4,
               weight=1.0, method=BEULER):
    """Single-compartment HH cells, one hsolve per cell, each with an
    excitatory and an inhibitory synchan and a spikegen.

    Returns (models, synapses) where synapses is a dict of CSR arrays over
    source cells: start, target cell, target synchan ('E' -> child 2,
    'I' -> child 3 in creation order), weight, delay steps."""
    rng = np.random.default_rng(seed)
    erest = -0.065
    na, k = hh_channels(erest)
    soma_l = soma_d = 20e-6
    area = soma_l * PI * soma_d
    xarea = PI * (soma_d / 2) ** 2
    n_exc = int(round(n_cells * frac_exc))
    vm0 = rng.uniform(-0.07, -0.05, size=n_cells)
    models = []
    for i in range(n_cells):
        c = Compartment(Em=sli(erest), Rm=sli(0.33 / area), Cm=sli(0.01 * area),
                        Ra=sli(0.3 * soma_l / xarea), initVm=float(vm0[i]), inject=0.0)
        c.children = [TabChannel(na, Gbar=sli(1200.0 * area)), TabChannel(k, Gbar=sli(360.0 * area)),
                      SynChan(tau1=5e-3, tau2=1e-3, gmax=6e-9, Ek=0.0),
                      SynChan(tau1=10e-3, tau2=1e-3, gmax=67e-9, Ek=-0.08),
                      SpikeGen(thresh=0.0, abs_refract=2e-3)]
        models.append(Model([c], dt=sli(dt), method=method))
    conn = rng.random((n_cells, n_cells)) < p_conn
    np.fill_diagonal(conn, False)
    start = [0]
    tgt, chan = [], []
    for src in range(n_cells):
        t = np.nonzero(conn[src])[0]
        tgt += t.tolist()
        chan += [2 if src < n_exc else 3] * len(t)
        start.append(len(tgt))
    dsteps = int((f32(delay) / sli(dt)) + 0.9)
    syn = dict(start=np.array(start, np.int32), target=np.array(tgt, np.int32),
               child_pos=np.array(chan, np.int32),
               weight=np.full(len(tgt), f32(weight)), delay_steps=np.full(len(tgt), dsteps, np.int32))
    return models, syn


# --------------------------------------------------------------------------
# Fast construction of many identical neurons
# --------------------------------------------------------------------------
def replicate(h, n, inject=None, vm=None):
    """``n`` one-neuron hsolves that share every array of ``h`` except chip[]
    (per-neuron inject current, compartment row 0's chip[1] slot of the soma)
    and vm. Equivalent to building each copy with :func:`model.build`.

    ``inject``: per-neuron values written into the soma's inject slot."""
    import copy
    soma = h.ncompts - 1                      # the root is the last row
    slot = int(h.compchips[soma]) + 1         # chip layout: Em/Rm, inject, ...
    out = []
    for i in range(n):
        c = copy.copy(h)
        if inject is not None:
            chip = h.chip.copy()
            chip[slot] = f32(inject[i])
            c.chip = chip
        if vm is not None:
            c.vm = np.full_like(h.vm, vm[i]) if np.ndim(vm[i]) == 0 else np.asarray(vm[i])
        out.append(c)
    return out


def inject_slot(h):
    """chip[] index of the soma's inject current in a one-neuron hsolve."""
    return int(h.compchips[h.ncompts - 1]) + 1


def cables_replicated(n_neurons, ncomp=16, seed=0, dt=20e-6, method=BEULER, gk_dend=0.0,
                      inject_range=(0.1e-9, 0.5e-9), erest=-0.065):
    """Configs 0/3 as one hsolve per neuron, built once and replicated."""
    rng = np.random.default_rng(seed)
    injects = rng.uniform(inject_range[0], inject_range[1], size=n_neurons)
    na, k = hh_channels(erest)
    from .model import build
    h = build(Model(cable_neuron(na, k, float(injects[0]), ncomp, erest=erest, gk_dend=gk_dend),
                    dt=sli(dt), method=method))
    return replicate(h, n_neurons, inject=[sli(x) for x in injects]), injects


def network_synapses(hs, syn):
    """Synapse table of :func:`hh_network` in the engine's and the oracle's
    terms: the target is the SYN2_OP of the target cell's synchan (its ops[]
    index), and, for the oracle, that synchan's child index."""
    n = len(hs)
    tgt_op = np.empty(len(syn["target"]), dtype=np.int32)
    tgt_child = np.empty(len(syn["target"]), dtype=np.int32)
    for k, (t, pos) in enumerate(zip(syn["target"], syn["child_pos"])):
        h = hs[t]
        cidx = h.syn_child[(0, int(pos))]
        tgt_child[k] = cidx
        tgt_op[k] = h.childops[cidx]
    return dict(src_start=syn["start"].astype(np.int64), target_solver=syn["target"].astype(np.int32),
                target_op=tgt_op, weight=syn["weight"], delay_steps=syn["delay_steps"]), tgt_child


# --------------------------------------------------------------------------
# Adjoint gradients (config 4)
# --------------------------------------------------------------------------
class GradTree:
    """Physical parameters of one config-4 neuron: a seeded random binary
    tree whose every compartment carries HH Na and K tabchannels and a leak
    (conductance gl through the membrane resistance). Parameters: per
    compartment gna, gk, gl (S/m^2); per neuron cm (F/m^2) and ra (ohm m).
    Geometry, inject and reversal potentials are fixed."""

    def __init__(self, parents, length, diam, gna, gk, gl, cm, ra, inject, erest=-0.065):
        self.parents = list(parents)
        self.length = np.asarray(length, dtype=np.float64)
        self.diam = np.asarray(diam, dtype=np.float64)
        self.gna = np.array(gna, dtype=np.float64)
        self.gk = np.array(gk, dtype=np.float64)
        self.gl = np.array(gl, dtype=np.float64)
        self.cm = float(cm)
        self.ra = float(ra)
        self.inject = float(inject)
        self.erest = float(erest)

    @property
    def area(self):
        return self.length * PI * self.diam

    @property
    def xarea(self):
        return PI * (self.diam / 2) ** 2

    def copy(self):
        return GradTree(self.parents, self.length, self.diam, self.gna, self.gk, self.gl, self.cm, self.ra,
                        self.inject, self.erest)

    def vector(self):
        """Parameters as one flat vector: gna, gk, gl (per compartment), cm, ra."""
        return np.concatenate([self.gna, self.gk, self.gl, [self.cm, self.ra]])

    def with_vector(self, v):
        n = len(self.parents)
        return GradTree(self.parents, self.length, self.diam, v[:n], v[n:2 * n], v[2 * n:3 * n], v[3 * n],
                        v[3 * n + 1], self.inject, self.erest)

    def model(self, na, k, dt=25e-6, method=BEULER) -> Model:
        """Compartments with fields computed in double (no SLI or float
        rounding): build with ``model.build(m, exact=True)``."""
        area, xarea = self.area, self.xarea
        comps = []
        for c, p in enumerate(self.parents):
            comp = Compartment(Em=self.erest, Rm=1.0 / (self.gl[c] * area[c]), Cm=self.cm * area[c],
                               Ra=self.ra * self.length[c] / xarea[c], initVm=self.erest,
                               inject=self.inject if c == 0 else 0.0, parent=p)
            comp.children = [TabChannel(na, Gbar=self.gna[c] * area[c]), TabChannel(k, Gbar=self.gk[c] * area[c])]
            comps.append(comp)
        return Model(comps, dt=dt, method=method)


def grad_trees(n_neurons=4096, ncomp=64, seed=4, soma=(30e-6, 30e-6), dend_len=20e-6,
               dia_range=(0.5e-6, 3e-6), inject_range=(0.2e-9, 0.6e-9)):
    """Config 4 neurons (seeded). Soma gna 1200, gk 360 S/m^2, dendrites a
    tenth of that, gl = 1/0.33 S/m^2, each scaled by U(0.8, 1.2) per
    compartment; cm = 0.01 F/m^2 x U(0.9, 1.1), ra = 0.3 ohm m x U(0.9, 1.1)
    per neuron. Returns (trees, (na, k) channel types)."""
    rng = np.random.default_rng(seed)
    na, k = hh_channels(-0.065)
    trees = []
    for _ in range(n_neurons):
        parents = random_binary_tree(rng, ncomp)
        length = np.full(ncomp, dend_len)
        diam = rng.uniform(*dia_range, size=ncomp)
        length[0], diam[0] = soma
        scale = np.where(np.arange(ncomp) == 0, 1.0, 0.1)
        gna = 1200.0 * scale * rng.uniform(0.8, 1.2, ncomp)
        gk = 360.0 * scale * rng.uniform(0.8, 1.2, ncomp)
        gl = (1.0 / 0.33) * rng.uniform(0.8, 1.2, ncomp)
        cm = 0.01 * rng.uniform(0.9, 1.1)
        ra = 0.3 * rng.uniform(0.9, 1.1)
        trees.append(GradTree(parents, length, diam, gna, gk, gl, cm, ra, rng.uniform(*inject_range)))
    return trees, (na, k)


def grad_targets(trees, seed=5, spread=0.2):
    """Target models: every gbar (Na, K, leak) scaled by U(1-spread, 1+spread)."""
    rng = np.random.default_rng(seed)
    out = []
    for t in trees:
        u = t.copy()
        n = len(t.parents)
        u.gna = t.gna * (1.0 + rng.uniform(-spread, spread, n))
        u.gk = t.gk * (1.0 + rng.uniform(-spread, spread, n))
        u.gl = t.gl * (1.0 + rng.uniform(-spread, spread, n))
        out.append(u)
    return out


def chip_roles(h):
    """Role of every chip[] entry of a one-tree solver built from
    :class:`GradTree`: ('emrm'|'inject'|'tbyc'|'diag', compt) or
    ('ek'|'gbar'|'state', compt, reversal potential of the channel). SETUP
    orders a compartment's channels by its own rules; the reversal potential
    identifies the channel."""
    from .model import (ADD_CURR_OP, CHAN_EK_OP, CHAN_OP, IPOL1V_OP, LCOMPT_OP, NEWVOLT_OP)
    roles = [None] * len(h.chip)
    ops = h.ops
    o = c = row = 0
    ek = 0.0
    while True:
        code = int(ops[o])
        o += 1
        if code == LCOMPT_OP:
            break
        elm = int(h.elmnum[row])
        roles[c], roles[c + 1] = ("emrm", elm), ("inject", elm)
        c += 2
        while int(ops[o]) > LCOMPT_OP:
            k = int(ops[o])
            o += 1
            if k == NEWVOLT_OP or k == ADD_CURR_OP:
                continue
            if k == CHAN_EK_OP:
                ek = float(h.chip[c])
                roles[c], roles[c + 1] = ("ek", elm, ek), ("gbar", elm, ek)
                c += 2
            elif k == CHAN_OP:   # keeps the previous channel's Ek
                roles[c] = ("gbar", elm, ek)
                c += 1
            elif k == IPOL1V_OP:
                o += 2
                roles[c] = ("state", elm, ek)
                c += 1
            else:
                raise ValueError("opcode %d outside the config-4 program" % k)
        roles[c], roles[c + 1] = ("tbyc", elm), ("diag", elm)
        c += 2
        row += 1
    return roles


def param_gradient(tree: GradTree, h, dchip, dravals, ena, dt=25e-6, method=BEULER):
    """Chain rule from the gradient with respect to one solver's chip[] and
    ravals[] to the tree's physical parameters (same order as
    ``GradTree.vector``), for arrays built with ``exact=True``:
      Gbar = g*area;  Em/Rm = Em*gl*area;  dt'/Cm = dt'/(cm*area);
      diag = 1 + dt'*gl/cm + coupling,  coupling and every ravals entry
      proportional to 1/(cm*ra);  dt' = dt/2 for Crank-Nicolson.
    ``ena`` is the Na channel's reversal potential (the other channel is K)."""
    n = len(tree.parents)
    dtc = dt / 2.0 if method == CRANK else dt
    area = tree.area
    g = np.zeros(3 * n + 2)
    for idx, role in enumerate(chip_roles(h)):
        kind, elm = role[0], role[1]
        d = float(dchip[idx])
        if kind == "gbar":
            g[(0 if abs(role[2] - ena) < 1e-12 else 1) * n + elm] += d * area[elm]
        elif kind == "emrm":
            g[2 * n + elm] += d * tree.erest * area[elm]
        elif kind == "tbyc":
            g[3 * n] += d * (-h.chip[idx] / tree.cm)
        elif kind == "diag":
            leak = dtc * tree.gl[elm] / tree.cm
            coupling = h.chip[idx] - 1.0 - leak
            g[2 * n + elm] += d * dtc / tree.cm
            g[3 * n] += d * (-(h.chip[idx] - 1.0) / tree.cm)
            g[3 * n + 1] += d * (-coupling / tree.ra)
    r = np.asarray(h.ravals, dtype=np.float64)
    dr = np.asarray(dravals[:len(r)], dtype=np.float64)
    g[3 * n] += float(np.dot(dr, -r / tree.cm))
    g[3 * n + 1] += float(np.dot(dr, -r / tree.ra))
    return g
