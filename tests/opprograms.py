"""Hand-assembled opcode programs shared by the opcode tests and the
fixture generator (tests/golden/make_golden.py).

Each program is one hsolve's flat arrays (ops[], chip[], tables, conc ...)
built by ophelpers, for opcodes and table kinds the benchmark models do not
produce. MODES are the three step paths the reference compiles: chanmode 4
with interpolation (hines_4chip.c), chanmode 5 under Crank-Nicolson, and
calcmode 0 (hines_4nichip.c). Opcode values follow
genesis/src/hines/hines_defs.h:178-222.
"""
import hashlib

import numpy as np

import ophelpers as A

DT = 2e-5


def _c(vm0=-0.062, inj=1e-10):
    # Em/Rm, inject, tbyc, diagterm, Rm, initial Vm
    return A.Compt(-0.065 / 3e8, inj, DT / 1e-11, 1.0 + DT / (1e-11 * 3e8), 3e8, vm0)


def prog_hh_like():
    c = _c()
    c.op(A.NEWVOLT).op(A.CHAN_EK, chips=[0.05, 1e-8]).op(A.IPOL1V, 0, 3, chips=[0.1])
    c.op(A.IPOL1V, 2, 1, chips=[0.6]).op(A.ADD_CURR, giv=3)
    c.op(A.CHAN_EK, chips=[-0.08, 3e-8]).op(A.IPOL1V, 4, 4, chips=[0.3]).op(A.ADD_CURR, giv=3)
    return [c], dict(tabs=A.tables(12, 40)), False


def prog_instant_powers():
    c = _c()
    c.op(A.NEWVOLT).op(A.CHAN_EK, chips=[0.02, 2e-8]).op(A.IPOL1V, 0, -2, chips=[0.2])
    c.op(A.IPOL1V, 2, 5, chips=[0.4]).op(A.IPOL1V, 4, 6, chips=[0.5]).op(A.ADD_CURR, giv=3)
    return [c], dict(tabs=A.tables(12, 40, seed=1)), False


def prog_chan_carry_two_compartments():
    c0 = _c(-0.06)
    c0.op(A.NEWVOLT).op(A.CHAN_EK, chips=[-0.07, 1e-8]).op(A.IPOL1V, 0, 2, chips=[0.3]).op(A.ADD_CURR, giv=3)
    c0.op(A.CHAN, chips=[2e-8]).op(A.IPOL1V, 2, 1, chips=[0.5]).op(A.ADD_CURR, giv=3)
    c1 = _c(-0.064)
    c1.op(A.NEWVOLT).op(A.CHAN, chips=[3e-8]).op(A.IPOL1V, 4, 3, chips=[0.2]).op(A.ADD_CURR, giv=3)
    return [c0, c1], dict(tabs=A.tables(12, 40, seed=2), parents=[1, -1]), False


def prog_tabcurrent():
    c = _c()
    c.op(A.NEWVOLT).op(A.CHAN_EK, chips=[0.0, 1e-8]).op(A.IPOL1V, 0, 2, chips=[0.3]).op(A.ADD_CURR, giv=3)
    c.op(A.CHAN, chips=[5e-9]).op(A.IPOL1V, 6, 0, giv=3)          # tabcurrent: current added at once
    c.op(A.CHAN_EK, chips=[-0.08, 1e-8]).op(A.IPOL1V, 8, 1, chips=[0.4]).op(A.ADD_CURR, giv=3)
    return [c], dict(tabs=A.tables(12, 40, seed=3)), False


def prog_nernst():
    c = _c()
    c.op(A.NEWVOLT).op(A.CONC_VAL, 0).op(A.NERNST, chips=[0.0125, 2e-8]).op(A.IPOL1V, 0, 2, chips=[0.3])
    c.op(A.ADD_CURR, giv=3)
    return [c], dict(tabs=A.tables(12, 40, seed=4), conc=[5e-5, 2.0]), True


def prog_ghk_same_ghk_flux():
    c = _c()
    c.op(A.NEWVOLT).op(A.CONC_VAL, 0).op(A.GHK, chips=[2 * 96485.3 / (8.314 * 300), 2 * 96485.3, 1e-12])
    c.op(A.IPOL1V, 0, 2, chips=[0.3]).op(A.ADD_CURR, giv=3).op(A.FLUX)
    c.op(A.SAME_GHK, chips=[2e-12]).op(A.IPOL1V, 2, 1, chips=[0.4]).op(A.ADD_CURR, giv=3)
    return [c], dict(tabs=A.tables(12, 40, seed=5), conc=[5e-5, 2.0]), True


def prog_tabghk():
    c = _c()
    c.op(A.NEWVOLT).op(A.DO_TABGHK).op(A.IPOL1V, 0, 0)
    c.op(A.SAME_GHK, chips=[3e-9]).op(A.IPOL1V, 2, 2, chips=[0.3]).op(A.ADD_CURR, giv=3)
    return [c], dict(tabs=A.tables(12, 40, seed=6)), False


def prog_domain():
    # DOMAIN_OP is emitted for a channel whose Ca domain feeds a concentration
    # gate; the solver then holds concentrations, which is what gives it a
    # concentration axis (hines_chip.c:131-140 sets yvals only when nconcs > 0)
    c = _c()
    c.op(A.NEWVOLT).op(A.CONC_VAL, 0).op(A.CHAN_EK, chips=[0.1, 1e-8]).op(A.IPOL1V, 0, 2, chips=[0.3])
    c.op(A.ADD_CURR, giv=3).op(A.FLUX)
    c.op(A.DOMAIN, chips=[1e7]).op(A.CHAN_EK, chips=[-0.08, 2e-8]).op(A.IPOL1C, 4, 1, chips=[0.2])
    c.op(A.ADD_CURR, giv=3)
    kw = dict(tabs=A.tables(12, 40, seed=7, ydivs=40), conc=[1e-4],
              concops=[A.CACONC, 0, A.LCACONC], concchip=[5e-5, 1.0 + DT / 0.04, DT * 3e11])
    return [c], kw, False


def prog_conc_gate_pool():
    c = _c()
    c.op(A.CONC_VAL, 0).op(A.NEWCONC1).op(A.NEWVOLT).op(A.CHAN_EK, chips=[-0.08, 1e-8])
    c.op(A.IPOL1V, 0, 1, chips=[0.3]).op(A.IPOL1C, 2, 2, chips=[0.2]).op(A.ADD_CURR, giv=3)
    c.op(A.CHAN_EK, chips=[0.12, 5e-9]).op(A.IPOL1V, 4, 2, chips=[0.1]).op(A.ADD_CURR, giv=3).op(A.FLUX)
    kw = dict(tabs=A.tables(12, 40, seed=8, ydivs=40, ymax=0.5), conc=[1e-4],
              concops=[A.CACONC, 0, A.LCACONC], concchip=[5e-5, 1.0 + DT / 0.04, DT * 3e11])
    return [c], kw, False


def prog_2d_tables():
    c = _c()
    c.op(A.CONC_VAL, 0).op(A.NEWCONC1).op(A.NEWVOLT).op(A.CHAN_EK, chips=[-0.08, 1e-8])
    c.op(A.IPOL2V, 0, 2, chips=[0.3]).op(A.ADD_CURR, giv=3)
    c.op(A.NEWCONC2, 1).op(A.CHAN_EK, chips=[0.05, 2e-9]).op(A.IPOL2C, 4, 1, chips=[0.4]).op(A.ADD_CURR, giv=3)
    return [c], dict(tabs=A.tables(30, 10, seed=9, ydivs=10, ymax=0.5), conc=[0.17, 0.31]), False


def prog_syn_mgblock():
    c = _c()
    xc2, yc1, yc2, xc1 = 0.99, 9.5e-5, 0.98, 9.9e-5
    c.op(A.CHAN_EK, chips=[0.0, 1e-9]).op(A.SYN2, 0, -1, 1, chips=[0.4, 0.7])
    c.op(A.MGBLOCK, chips=[0.3, 1 / 0.062, 1.2], giv=6)           # blocked and unblocked currents
    return [c], dict(tabs=A.tables(12, 40), stablist=[xc2, yc1, yc2, xc1 / DT]), True


def prog_elmmpump():
    c = _c()
    c.op(A.CONC_VAL, 0).op(A.ELMMPUMP, chips=[2e-4, 3e-12, 1e-3], giv=1)
    c.op(A.NEWVOLT).op(A.CHAN_EK, chips=[-0.08, 1e-8]).op(A.IPOL1V, 0, 2, chips=[0.3]).op(A.ADD_CURR, giv=3)
    return [c], dict(tabs=A.tables(12, 40, seed=10), conc=[1e-4]), False


def prog_spike():
    c = _c(-0.02, 5e-9)
    c.op(A.NEWVOLT).op(A.SPIKE, 0, 5, chips=[-0.03]).op(A.CHAN_EK, chips=[-0.08, 1e-8])
    c.op(A.IPOL1V, 0, 2, chips=[0.3]).op(A.ADD_CURR, giv=3)
    return [c], dict(tabs=A.tables(12, 40, seed=11)), False


PROGRAMS = {f.__name__[5:]: f for f in (
    prog_hh_like, prog_instant_powers, prog_chan_carry_two_compartments, prog_tabcurrent, prog_nernst,
    prog_ghk_same_ghk_flux, prog_tabghk, prog_domain, prog_conc_gate_pool, prog_2d_tables, prog_syn_mgblock,
    prog_elmmpump, prog_spike)}


MODES = ((4, 1, False), (5, 1, True), (4, 0, False))
NSTEPS = 400


def build(name, chanmode=4, calcmode=1, crank=False):
    """The program's arrays in one step mode; also whether it calls libm."""
    compts, kw, libm = PROGRAMS[name]()
    tabs = kw.pop("tabs")
    h = A.solver(compts, tabs, dt=DT, chanmode=chanmode, calcmode=calcmode, crank=crank, **kw)
    return h, libm


def mode_tag(name, chanmode, calcmode, crank):
    return "%s/cm%d_calc%d_cn%d" % (name, chanmode, calcmode, int(crank))


def input_digest(h):
    """sha256 over the arrays and scalars of one solver's description."""
    m = hashlib.sha256()
    for k in ("ops", "chip", "funcs", "ravals", "vm", "givals", "tablist", "xvals", "yvals", "stablist", "conc",
              "concops", "concchip"):
        m.update(np.ascontiguousarray(getattr(h, k)).tobytes())
    m.update(np.array([h.ncompts, h.ncols, h.xdivs, h.xmin, h.invdx, h.ydivs, h.ymin, h.invdy, h.dt, h.crank,
                       h.chanmode, h.calcmode], dtype=np.float64).tobytes())
    diff = getattr(h, "diff", None)
    if diff is not None:
        for k in sorted(diff):
            m.update(np.ascontiguousarray(diff[k], dtype=np.float64).tobytes())
    return m.hexdigest()


ARRAYS = ("ops", "chip", "funcs", "ravals", "vm", "givals", "tablist", "xvals", "yvals", "stablist", "conc",
          "concops", "concchip", "childops", "childchips")
SCALARS = ("ncompts", "ncols", "xdivs", "xmin", "invdx", "ydivs", "ymin", "invdy", "dt", "crank", "chanmode",
           "calcmode", "method")


def to_fixture(h, tag, out):
    """Stores one solver's input arrays under tag/in/... (numpy's sin/cos,
    used to build the tables, may round differently on another machine, so
    the fixture carries the exact inputs the reference stepped)."""
    for k in ARRAYS:
        out[tag + "/in/" + k] = np.asarray(getattr(h, k))
    out[tag + "/in/scalars"] = np.array([float(getattr(h, k)) for k in SCALARS])


def from_fixture(d, tag):
    """The solver whose inputs to_fixture stored."""
    from types import SimpleNamespace
    kw = {k: d[tag + "/in/" + k] for k in ARRAYS}
    sc = d[tag + "/in/scalars"]
    for k, v in zip(SCALARS, sc):
        kw[k] = float(v) if k in ("xmin", "invdx", "ymin", "invdy", "dt") else int(v)
    return SimpleNamespace(diff=None, **kw)


def syn_countdown_words(ops):
    """Positions of the SYN2_OP/SYN3_OP countdown words in ops[] (the word
    after the stablist index). The reference keeps each synchan's time to
    its next event there, set by HSEVENT and h_dosynchan (hines.c:352-357,
    hines_conn.c:62-89); the engine keeps its events in per-step rings
    instead and does not maintain this word."""
    ops = np.asarray(ops)
    out = []
    i = 0
    while i < len(ops) and ops[i] != A.LCOMPT:
        if ops[i] in (A.SYN2, A.SYN3):
            out.append(i + 2)
            i += 4
        else:
            i += 1
    return np.array(out, dtype=np.int64)


def syn3_solver(p_fire, stablist, n_compts=1, seed_vm=-0.062):
    """Compartments each with one SYN3_OP synchan (randomly triggered,
    channelC3): chip layout per compartment [Em/Rm, inject, Ek, gmax,
    dt*frequency, X, Y, dt/Cm, diagonal term]; X sits at 9 * c + 5."""
    comps = []
    for c in range(n_compts):
        cc = _c(seed_vm)
        # a synapse op adds its channel's current itself (hines_chip.c:551-567)
        cc.op(A.CHAN_EK, chips=[0.0, 1e-9]).op(A.SYN3, 0, -1, 1, chips=[p_fire, 0.0, 0.0], giv=3)
        comps.append(cc)
    return A.solver(comps, A.tables(12, 40), dt=DT, stablist=stablist)
