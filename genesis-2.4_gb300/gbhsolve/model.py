"""Model description and SETUP restatement for GENESIS ``hsolve`` chanmode 4/5.

The engine consumes the flat arrays the reference ``hsolve`` builds at SETUP
(``ops[]``, ``chip[]``, ``funcs[]``, ``ravals[]``, ``tablist[]``, ``concops[]``,
``concchip[]`` ...).  Inside GENESIS those arrays come from the reference's own
setup code; this module restates that code for the element types the benchmark
models use, so that the same arrays can be produced without a GENESIS build:

* ``compartment`` (asymmetric, AXIAL/RAXIAL)      -- hines_init.c:40-345
* ``tabchannel`` X/Y voltage gates, Z voltage or Ca-dependent gate
                                                   -- hines_chip_init.c:465-1260
* ``Ca_concen`` fed by ``I_Ca`` from a channel     -- hines_conc_init.c:477-800
* ``synchan`` receiving spike events               -- hines_chip_init.c:855-890
* ``spikegen``                                     -- hines_chip_init.c:745-752
* child classification and ordering                -- hines_child.c:81-1549, 1998-2090
* composite table with the trapezoid transform     -- hines_chip_init.c:1262-1400
* element fields -> chip[] (RESET)                 -- hines_chip_init.c:1402-1552,
                                                      hines_data.c:80-535
* elimination program funcs[]/ravals[]             -- hines_init.c:361-1273

Element fields that GENESIS stores as ``float`` are rounded to float32 on
assignment, exactly as the reference structs do (segment/seg_struct.h:209-221,
olf/olf_struct.h:142-155, sim/struct_defs.h:118-134).
"""
from __future__ import annotations

import math
import pickle
import struct
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# opcode values (hines_defs.h:178-222)
TABCURR_OP, COMPT_OP, FCOMPT_OP, LCOMPT_OP = 0, 100, 101, 102
SPIKE_OP, ELMMPUMP_OP, CONC_VAL_OP, NERNST_OP, GHK_OP = 200, 500, 1000, 2000, 2010
CHAN_OP, CHAN_EK_OP, SAME_GHK_OP, DO_TABGHK_OP = 3000, 3001, 3002, 3003
ADD_CURR_OP, FLUX_OP, SCALE_FLUX_OP = 3200, 3300, 3301
STORE_ALL_OP, STORE_ALLI_OP, STORE_ALLC_OP = 3500, 3501, 3502
IPOL1V_OP, IPOL1C_OP, IPOL2V_OP, IPOL2C_OP = 4001, 4002, 4003, 4004
SYN2_OP, SYN3_OP, MGBLOCK_OP = 4100, 4101, 4200
NEWVOLT_OP, NEWCONC1_OP, NEWCONC2_OP, DOMAIN_OP = 5100, 5110, 5111, 5112
CACONC_OP, LCACONC_OP = 10200, 10202
# funcs codes (hines_defs.h:120-128)
FORWARD_ELIM, SET_DIAG, SKIP_DIAG, CALC_RESULTS, FINISH = 0, 1, 2, 6, 7
# child types (hines_defs.h:130-165)
SPIKEGEN_T, TABCHAN_T, SYNCHANC_T, CACONCEN_T = 11, 20, 32, 50

BEULER, CRANK = 10, 11          # integration method codes (sim_defs.h:174-175)
TINY, VTINY = 1.0e-6, 1.0e-10   # hines_defs.h
SING_TINY = 1e-6                # olf_defs.h:58
MAXTABC = 40                    # first voltage-table slot (hines_defs.h:59)


_F32 = struct.Struct("f")


def f32(x: float) -> float:
    """Value as stored in a GENESIS ``float`` field (IEEE single, round to
    nearest even, as the C double-to-float conversion does)."""
    return _F32.unpack(_F32.pack(x))[0]


_f32_field = f32


def sli(x: float) -> float:
    """Value after an SLI expression is passed as a command argument: SLI
    formats floats with ``%0.10g`` (sim/sim_main.c:372, ss/eval.c:1075)."""
    return float("%0.10g" % x)


# --------------------------------------------------------------------------
# Interpolation tables (olf/new_interp.c)
# --------------------------------------------------------------------------
class Interpol:
    """``Interpol`` struct created by ``create_interpol`` (new_interp.c:275-297)."""

    def __init__(self, xdivs: int, xmin: float, xmax: float):
        self.xdivs = int(xdivs)
        self.xmin = float(xmin)
        self.xmax = float(xmax)
        self.table = np.zeros(self.xdivs + 1, dtype=np.float64)
        self.dx = (self.xmax - self.xmin) / float(self.xdivs)
        self.invdx = 1.0 / self.dx if abs(self.dx) > 1e-50 else 1.0

    def interp(self, x: float) -> float:
        """``TabInterp`` in LIN_INTERP mode (new_interp.c:242-256)."""
        lo = (x - self.xmin) * self.invdx
        if lo <= 0.0:
            return float(self.table[0])
        if lo >= self.xdivs:
            return float(self.table[self.xdivs])
        ilo = int(lo)
        xv = float(self.table[ilo])
        return (lo - float(ilo)) * (float(self.table[ilo + 1]) - xv) + xv


def setup_alpha(args, xdivs=3000, xmin=-0.1, xmax=0.05):
    """``setupalpha`` (new_interp.c:533-580 with mode SETUP_ALPHA): returns
    the (A, B) tables, B holding alpha+beta.  ``args`` are the ten rate
    constants AA AB AC AD AF BA BB BC BD BF as doubles."""
    a = [float(v) for v in args]
    A = Interpol(xdivs, xmin, xmax)
    B = Interpol(xdivs, xmin, xmax)
    dx = (xmax - xmin) / xdivs
    x = xmin
    for i in range(xdivs + 1):
        if abs(a[4]) < SING_TINY:
            temp = 0.0
        else:
            t2 = a[2] + math.exp((x + a[3]) / a[4])
            temp = float(A.table[i - 1]) if abs(t2) < SING_TINY else (a[0] + a[1] * x) / t2
        A.table[i] = temp
        if abs(a[9]) < SING_TINY:
            bv = 0.0
        else:
            t2 = a[7] + math.exp((x + a[8]) / a[9])
            bv = float(B.table[i - 1]) if abs(t2) < SING_TINY else (a[5] + a[6] * x) / t2
        B.table[i] = bv + temp
        x += dx
    return A, B


def setup_tau_table(tau_minf, xdivs=3000, xmin=-0.1, xmax=0.05):
    """Tables filled directly from tau(x) and minf(x) callables the way
    ``tweak``-style scripts do (A = minf/tau, B = 1/tau); used for the Ca
    dependent gates whose axis is a concentration."""
    A = Interpol(xdivs, xmin, xmax)
    B = Interpol(xdivs, xmin, xmax)
    dx = (xmax - xmin) / xdivs
    x = xmin
    for i in range(xdivs + 1):
        tau, minf = tau_minf(x)
        A.table[i] = minf / tau
        B.table[i] = 1.0 / tau
        x += dx
    return A, B


@dataclass
class GateTables:
    A: Interpol
    B: Interpol


@dataclass
class ChannelType:
    """A ``tabchannel`` prototype in /library; copies share its tables."""
    name: str
    Ek: float
    Xpower: float = 0.0
    Ypower: float = 0.0
    Zpower: float = 0.0
    X: Optional[GateTables] = None
    Y: Optional[GateTables] = None
    Z: Optional[GateTables] = None
    Z_conc: bool = False
    instant: int = 0


# --------------------------------------------------------------------------
# Elements
# --------------------------------------------------------------------------
@dataclass
class TabChannel:
    ctype: ChannelType
    Gbar: float
    Ek: Optional[float] = None        # defaults to the prototype's Ek
    conc_src: Optional[int] = None    # index (in the compartment's children) of
                                      # the Ca_concen sending CONCEN (Z_conc gate)
    flux_to: Optional[int] = None     # index of the Ca_concen receiving I_Ca


@dataclass
class CaConcen:
    tau: float
    B: float
    Ca_base: float
    thick: float = 0.0


@dataclass
class SynChan:
    tau1: float
    tau2: float
    gmax: float
    Ek: float
    nsynapses: int = 0


@dataclass
class SpikeGen:
    thresh: float
    abs_refract: float


@dataclass
class Compartment:
    Em: float
    Rm: float
    Cm: float
    Ra: float
    initVm: float
    inject: float = 0.0
    parent: int = -1                  # index into the model's compartment list
    children: List[object] = field(default_factory=list)  # creation order


@dataclass
class Model:
    """An hsolve: compartments listed in the order the ``path`` wildcard
    returns them (element creation order)."""
    compartments: List[Compartment]
    dt: float
    method: int = BEULER
    chanmode: int = 4
    calcmode: int = 1


# --------------------------------------------------------------------------
# Arrays produced by SETUP + RESET
# --------------------------------------------------------------------------
@dataclass
class HsolveArrays:
    ncompts: int
    ops: np.ndarray
    chip: np.ndarray
    funcs: np.ndarray
    ravals: np.ndarray
    vm: np.ndarray
    givals: np.ndarray
    ncols: int
    xdivs: int
    xmin: float
    invdx: float
    tablist: np.ndarray      # (xdivs+2)*ncols: last row duplicates row xdivs
    xvals: np.ndarray        # xdivs+2 entries: last duplicates xvals[xdivs]
    ydivs: int
    ymin: float
    invdy: float
    yvals: np.ndarray
    stablist: np.ndarray
    conc: np.ndarray
    flux: np.ndarray
    concops: np.ndarray
    concchip: np.ndarray
    childops: np.ndarray
    childchips: np.ndarray
    compchips: np.ndarray
    compops: np.ndarray
    elmnum: np.ndarray       # row -> compartment index
    hnum: np.ndarray         # compartment index -> row
    parent_row: np.ndarray   # row -> parent row (-1 root)
    syn_child: dict          # (compartment index, child position) -> child index
    spike_op: np.ndarray     # row -> ops index of SPIKE_OP or -1
    dt: float
    method: int
    chanmode: int
    calcmode: int

    @property
    def crank(self) -> int:
        return 1 if self.method == CRANK else 0


def _hnum(parents, kids, ncompts):
    """do_hnum (hines_init.c:317-345) over every root in list order, then the
    per-parent bubble sort of kids by Hines number (hines_init.c:279-295)."""
    hnum = [0] * ncompts
    elmnum = [0] * ncompts
    counter = [ncompts - 1]

    def number(c):
        stack = [c]
        while stack:
            c = stack.pop()
            hnum[c] = counter[0]
            elmnum[counter[0]] = c
            counter[0] -= 1
            for k in kids[c]:
                if not kids[k]:
                    hnum[k] = counter[0]
                    elmnum[counter[0]] = k
                    counter[0] -= 1
            # recurse into kids with kids of their own, first one first
            for k in reversed([k for k in kids[c] if kids[k]]):
                stack.append(k)

    for i in range(ncompts):
        if parents[i] == -1:
            number(i)
    for c in range(ncompts):
        kids[c].sort(key=lambda k: hnum[k])
    return hnum, elmnum


def _child_sort(keys):
    """The per-compartment insertion sort of do_hget_children
    (hines_child.c:1264-1279): an element moves left past every element that
    does not compare as 'belongs before' it, so equal keys end up reversed."""
    idx = list(range(len(keys)))
    for j in range(1, len(idx)):
        temp = idx[j]
        m = j - 1
        while m >= 0 and not _belongs_before(keys[idx[m]], keys[temp]):
            idx[m + 1] = idx[m]
            m -= 1
        idx[m + 1] = temp
    return idx


def _belongs_before(a, b):
    """hchild_compare (hines_child.c:1998-2090) on precomputed keys
    (type, conc, Ek) for the supported child types."""
    ta, ca, ea = a
    tb, cb, eb = b
    if ta >= CACONCEN_T and tb >= CACONCEN_T:
        return False  # single pool per compartment in the supported subset
    if ta < tb:
        return True
    if ta == tb and ta == TABCHAN_T:
        if ca < cb:
            return True
        if ca == cb and ea < eb:
            return True
    return False


_TABLE_CACHE = {}


def build(model: Model, exact: bool = False) -> HsolveArrays:
    """SETUP + RESET of one hsolve over ``model``; returns the flat arrays.

    ``exact=True`` skips the rounding of element fields to float storage, so
    the arrays are smooth functions of the model's parameters (used by the
    differentiated form's finite-difference checks); the default reproduces
    the reference's arrays."""
    f32 = (lambda x: float(x)) if exact else _f32_field
    comps = model.compartments
    n = len(comps)
    dt = float(model.dt)
    crank = model.method == CRANK
    dtc = dt / 2.0 if crank else dt

    parents = [c.parent for c in comps]
    kids = [[] for _ in range(n)]
    for j in range(n):
        if parents[j] != -1:
            kids[parents[j]].append(j)
    hnum, elmnum = _hnum(parents, kids, n)

    # ---- children: classify, order (hines_child.c) ----
    # per row: list of (original child position, element)
    row_children = []
    for i in range(n):
        cp = comps[elmnum[i]]
        keys = []
        for pos, ch in enumerate(cp.children):
            if isinstance(ch, TabChannel):
                conc = 0
                if ch.conc_src is not None:
                    conc = ch.conc_src + 1
                elif ch.flux_to is not None:
                    conc = ch.flux_to + 1
                ek = f32(ch.ctype.Ek if ch.Ek is None else ch.Ek)
                keys.append((TABCHAN_T, conc, ek))
            elif isinstance(ch, SynChan):
                keys.append((SYNCHANC_T, 0, 0.0))
            elif isinstance(ch, SpikeGen):
                keys.append((SPIKEGEN_T, 0, 0.0))
            elif isinstance(ch, CaConcen):
                keys.append((CACONCEN_T, 0, 0.0))
            else:
                raise ValueError("unsupported child element %r" % type(ch))
        order = _child_sort(keys)
        row_children.append([(p, cp.children[p]) for p in order])
        if sum(1 for _, ch in row_children[-1] if isinstance(ch, SpikeGen)) > 1:
            raise ValueError("second spikegen in one hsolve compartment")

    # conc indices: one per Ca_concen, in row order (hines_child.c:1556-1596)
    conc_index = {}
    nconcs = 0
    for i in range(n):
        for p, ch in row_children[i]:
            if isinstance(ch, CaConcen):
                conc_index[(i, p)] = nconcs
                nconcs += 1

    # ---- composite table layout (check_tab, duplicate_tables) ----
    slots = {}            # slot -> (Interpol, integrate flag)
    nct, nvt = 0, MAXTABC
    gate_slot = {}        # (id(table B), flag) -> slot of B
    xdivs = ydivs = 0
    xmin = invdx = ymin = invdy = 0.0

    def check_tab(A: Interpol, B: Interpol, conc: bool, instant: bool):
        nonlocal nct, nvt, xdivs, ydivs, xmin, invdx, ymin, invdy
        flag = -1 if instant else 0
        key = (id(B), flag)
        if key in gate_slot:
            return gate_slot[key]
        for tab in (B, A):
            if conc:
                if ydivs == 0:
                    ydivs, ymin, invdy = tab.xdivs, tab.xmin, tab.invdx
                elif (tab.xdivs, tab.xmin, tab.invdx) != (ydivs, ymin, invdy):
                    raise ValueError("all concentration tables must have the same size")
            else:
                if xdivs == 0:
                    xdivs, xmin, invdx = tab.xdivs, tab.xmin, tab.invdx
                elif (tab.xdivs, tab.xmin, tab.invdx) != (xdivs, xmin, invdx):
                    raise ValueError("all voltage tables must have the same size")
        if conc:
            sb = nct
            nct += 2
        else:
            sb = nvt
            nvt += 2
        slots[sb] = (B, flag)
        slots[sb + 1] = (A, flag)
        gate_slot[key] = sb
        return sb

    chan_gates = {}  # (row, pos) -> list of (gate letter, slot, power)
    for i in range(n):
        for p, ch in row_children[i]:
            if not isinstance(ch, TabChannel):
                continue
            ct = ch.ctype
            gl = []
            for letter in "XYZ":
                gt = getattr(ct, letter)
                if gt is None:
                    continue
                pw = getattr(ct, letter + "power")
                if pw < 1 or pw > 6:
                    raise ValueError("gate power must be 1-6 for chanmode >= 2")
                inst = bool(ct.instant & {"X": 1, "Y": 2, "Z": 4}[letter])
                conc = letter == "Z" and ct.Z_conc
                sb = check_tab(gt.A, gt.B, conc, inst)
                power = int(pw + 1e-6)
                if inst:
                    power = -power
                gl.append((letter, sb, power, conc))
            chan_gates[(i, p)] = gl
    if xdivs and ydivs and xdivs != ydivs:
        raise ValueError("xdivs=%d while ydivs=%d" % (xdivs, ydivs))

    ntab = nct + nvt - MAXTABC
    ncols = ntab
    tabindex = {}
    tablist = np.zeros(0)
    xvals = np.zeros(0)
    yvals = np.zeros(0)
    # cells built from the same channel types at the same dt get the same
    # composite table: one shared (read-only) copy instead of one per cell
    tkey = (tuple((sl, id(t), fl) for sl, (t, fl) in sorted(slots.items())), xdivs, xmin, invdx, ydivs, ymin,
            invdy, dt)
    cached = _TABLE_CACHE.get(tkey) if ntab else None
    if cached is not None:
        tabindex, tablist, xvals, yvals = cached[0]
    elif ntab:
        tabsize = xdivs + 1
        if ydivs and not xdivs:
            tabsize = ydivs + 1
        tablist = np.zeros((tabsize + 1) * ncols, dtype=np.float64)
        xv = []
        x = xmin
        dxx = 1.0 / invdx if invdx else 0.0
        for _ in range(tabsize):
            xv.append(x)
            x += dxx
        xv.append(xv[-1])
        xvals = np.array(xv, dtype=np.float64)
        if ydivs:
            yv = []
            y = ymin
            dy = 1.0 / invdy
            for _ in range(ydivs + 1):
                yv.append(y)
                y += dy
            yv.append(yv[-1])
            yvals = np.array(yv, dtype=np.float64)
        tby2 = dt / 2.0
        col = 0
        for s in sorted(slots):
            if s % 2:
                continue
            B, flag = slots[s]
            A, _ = slots[s + 1]
            tabindex[s] = col
            if flag == 0:
                tablist[col:tabsize * ncols:ncols] = 1.0 + tby2 * B.table[:tabsize]
                tablist[col + 1:tabsize * ncols:ncols] = dt * A.table[:tabsize]
            else:
                tablist[col:tabsize * ncols:ncols] = B.table[:tabsize]
                tablist[col + 1:tabsize * ncols:ncols] = A.table[:tabsize]
            col += 2
        # padding row: the reference reads one row past the end when the
        # index is clamped to xdivs; a copy keeps that read finite.
        tablist[tabsize * ncols:] = tablist[(tabsize - 1) * ncols:tabsize * ncols]
        for a in (tablist, xvals, yvals):
            a.flags.writeable = False
        if len(_TABLE_CACHE) >= 64:
            _TABLE_CACHE.clear()
        # the Interpol objects are kept with the entry so their ids stay unique
        _TABLE_CACHE[tkey] = ((dict(tabindex), tablist, xvals, yvals), [t for t, _ in slots.values()])
    if ntab == 0:
        xmin = invdx = ymin = invdy = 0.0

    # synchan constants (check_stab, hines_chip_init.c:430-462)
    stab = []
    syn_const = {}
    for i in range(n):
        for p, ch in row_children[i]:
            if isinstance(ch, SynChan):
                t1, t2 = f32(ch.tau1), f32(ch.tau2)
                xc1 = t1 * (1.0 - math.exp(-dt / t1))
                xc2 = math.exp(-dt / t1)
                yc1 = t2 * (1.0 - math.exp(-dt / t2))
                yc2 = math.exp(-dt / t2)
                if t1 == t2:
                    norm = f32(ch.gmax) * math.e / t1
                else:
                    tpeak = t1 * t2 * math.log(t1 / t2) / (t1 - t2)
                    norm = f32(ch.gmax) * (t1 - t2) / (t1 * t2 * (math.exp(-tpeak / t1) - math.exp(-tpeak / t2)))
                norm = f32(norm)
                k = None
                for j in range(0, len(stab), 4):
                    if (abs(stab[j] - xc2) < VTINY and abs(stab[j + 1] - yc1) < VTINY and
                            abs(stab[j + 2] - yc2) < VTINY and
                            (abs(stab[j + 3] - xc1) < VTINY or abs(stab[j + 3] - xc1 / dt) < VTINY)):
                        k = j
                        break
                if k is None:
                    k = len(stab)
                    stab += [xc2, yc1, yc2, xc1 / dt]
                syn_const[(i, p)] = (k, norm)

    # ---- ops / chip (h_hh_chip_init fill pass + do_chip_hreset) ----
    ops: List[int] = []
    chip: List[float] = []
    compchips = np.zeros(n, dtype=np.int32)
    compops = np.zeros(n, dtype=np.int32)
    vm = np.zeros(n, dtype=np.float64)
    nchildren = sum(len(rc) for rc in row_children)
    childops = np.zeros(nchildren + 2, dtype=np.int32)
    childchips = np.zeros(nchildren + 2, dtype=np.int32)
    syn_child = {}
    spike_op = np.full(n, -1, dtype=np.int32)
    gate_init = {}
    last_ek = 1.0e30
    lastconc = -1
    child_idx = 1  # children are numbered from 1 (hines_child.c:194)
    for i in range(n):
        cp = comps[elmnum[i]]
        compops[i] = len(ops)
        compchips[i] = len(chip)
        ops.append(FCOMPT_OP if i == 0 else COMPT_OP)
        Em, Rm, Cm = f32(cp.Em), f32(cp.Rm), f32(cp.Cm)
        chip += [f32(f32(Em) / f32(Rm)), f32(cp.inject)]
        vm[i] = f32(cp.initVm)  # compartment RESET: Vm = initVm
        has_volt = any(isinstance(ch, TabChannel) and
                       any(not g[3] for g in chan_gates[(i, p)])
                       for p, ch in row_children[i])
        if has_volt:
            ops.append(NEWVOLT_OP)
        lastc1 = False
        for p, ch in row_children[i]:
            cidx = child_idx
            child_idx += 1
            if isinstance(ch, SpikeGen):
                childops[cidx] = len(ops)
                childchips[cidx] = len(chip)
                spike_op[i] = len(ops)
                # chip_put_spike: counter 0, refractory steps, threshold
                ops += [SPIKE_OP, 0, int((f32(ch.abs_refract) / dt) + 1.9)]
                chip.append(f32(ch.thresh))
            elif isinstance(ch, CaConcen):
                childops[cidx] = len(ops)
                childchips[cidx] = len(chip)
            elif isinstance(ch, TabChannel):
                gl = chan_gates[(i, p)]
                conc_gate = any(g[3] for g in gl)
                if conc_gate:
                    k = conc_index[(i, _child_pos(row_children[i], ch.conc_src))]
                    if k != lastconc:
                        ops += [CONC_VAL_OP, k]
                        lastconc = k
                    if not lastc1:
                        ops.append(NEWCONC1_OP)
                        lastc1 = True
                ek = f32(ch.ctype.Ek if ch.Ek is None else ch.Ek)
                if abs(ek - last_ek) < VTINY:
                    ops.append(CHAN_OP)
                    chip.append(f32(ch.Gbar))
                else:
                    ops.append(CHAN_EK_OP)
                    chip += [ek, f32(ch.Gbar)]
                    last_ek = ek
                childops[cidx] = len(ops)
                childchips[cidx] = len(chip)
                for letter, sb, power, conc in gl:
                    ops += [IPOL1C_OP if conc else IPOL1V_OP, tabindex[sb], power]
                    gate_init[(len(chip))] = (i, p, letter)
                    chip.append(0.0)  # filled at RESET below
                ops.append(ADD_CURR_OP)
                if ch.flux_to is not None:
                    k = conc_index[(i, _child_pos(row_children[i], ch.flux_to))]
                    if k != lastconc:
                        ops += [CONC_VAL_OP, k]
                        lastconc = k
                    ops.append(FLUX_OP)
            elif isinstance(ch, SynChan):
                k, norm = syn_const[(i, p)]
                ek = f32(ch.Ek)
                if abs(ek - last_ek) < VTINY:
                    ops.append(CHAN_OP)
                    chip.append(norm)
                else:
                    ops.append(CHAN_EK_OP)
                    chip += [ek, norm]
                    last_ek = ek
                childops[cidx] = len(ops)
                childchips[cidx] = len(chip)
                syn_child[(elmnum[i], p)] = cidx
                ops += [SYN2_OP, k, -1, cidx]
                chip += [0.0, 0.0]  # X, Y reset to zero
        chip += [dtc / Cm, 0.0]  # tbyc; diagterm filled by h_funcs_init
    ops.append(LCOMPT_OP)

    chip_arr = np.array(chip, dtype=np.float64)
    # gate states at RESET: X = A(Vm)/B(Vm) from the channel's own tables
    # (olf/tabchannel.c RESET) at the compartment's initVm, or at the pool's
    # initial concentration for a Z_conc gate.
    for slot, (i, p, letter) in gate_init.items():
        ch = row_children[i][[q for q, _ in row_children[i]].index(p)][1]
        gt = getattr(ch.ctype, letter)
        if letter == "Z" and ch.ctype.Z_conc:
            pool = comps[elmnum[i]].children[ch.conc_src]
            v = float(pool.Ca_base)
        else:
            v = vm[i]
        chip_arr[slot] = gt.A.interp(v) / gt.B.interp(v)

    # ---- funcs / ravals (h_funcs_init, asymmetric compartments) ----
    funcs: List[int] = []
    ravals: List[float] = []
    diagterms = np.zeros(n, dtype=np.float64)
    parent_row = np.full(n, -1, dtype=np.int32)
    for i in range(n):
        c = elmnum[i]
        if parents[c] >= 0:
            parent_row[i] = hnum[parents[c]]
    skipdiag = False
    for i in range(n):
        c = elmnum[i]
        cp = comps[c]
        Cm = f32(cp.Cm)
        diagterms[i] = 1.0 + dtc / (Cm * f32(cp.Rm))
        nk = len(kids[c])
        if skipdiag:
            skipdiag = False
        elif nk or parents[c] == -1:
            if i > 1:
                funcs.append(SET_DIAG)
        elif i > 1:
            funcs.append(SKIP_DIAG)
            skipdiag = True
        for k in kids[c]:
            link = comps[k]
            row = hnum[k]
            funcs += [FORWARD_ELIM, 2 * row]
            t = -dtc / (Cm * f32(link.Ra))
            ravals.append(t)
            diagterms[i] -= t
            # float*float: the product is formed in float (hines_init.c:734)
            t = -dtc / f32(f32(link.Cm) * f32(link.Ra))
            ravals.append(t)
            diagterms[row] -= t
    funcs.append(FINISH)
    for i in range(n - 2, -1, -1):
        c = elmnum[i]
        if parents[c] != -1:
            cp = comps[c]
            funcs += [FORWARD_ELIM, 2 * hnum[parents[c]]]
            ravals.append(-dtc / (f32(cp.Cm) * f32(cp.Ra)))
        funcs.append(CALC_RESULTS)
    funcs.append(FINISH)
    for i in range(n):
        j = len(chip_arr) - 1 if i == n - 1 else compchips[i + 1] - 1
        chip_arr[j] = diagterms[i]

    # ---- givals layout (hines_child.c:1497-1549): Rm, Ileak, 3/channel, Im ----
    gv = [0.0]
    for i in range(n):
        gv += [f32(comps[elmnum[i]].Rm), 0.0]
        for p, ch in row_children[i]:
            if isinstance(ch, (TabChannel, SynChan)):
                gv += [0.0, 0.0, 0.0]
        gv.append(0.0)
    givals = np.array(gv, dtype=np.float64)

    # ---- concentrations (h_init_conc_chip, chip_put_Ca_concen) ----
    conc = np.zeros(max(nconcs, 0), dtype=np.float64)
    concops: List[int] = []
    concchip: List[float] = []
    for i in range(n):
        for p, ch in row_children[i]:
            if isinstance(ch, CaConcen):
                k = conc_index[(i, p)]
                conc[k] = float(ch.Ca_base)
                concops += [CACONC_OP, k]
                tau = f32(ch.tau)
                concchip += [float(ch.Ca_base), 1.0 + dt / f32(2 * f32(tau)),
                             dt * f32(ch.B)]
    if nconcs:
        concops.append(LCACONC_OP)

    return HsolveArrays(
        ncompts=n,
        ops=np.array(ops, dtype=np.int32),
        chip=chip_arr,
        funcs=np.array(funcs, dtype=np.int32),
        ravals=np.array(ravals, dtype=np.float64),
        vm=vm,
        givals=givals,
        ncols=ncols,
        xdivs=xdivs if ntab else 0,
        xmin=xmin, invdx=invdx,
        tablist=tablist, xvals=xvals,
        ydivs=ydivs, ymin=ymin, invdy=invdy, yvals=yvals,
        stablist=np.array(stab, dtype=np.float64),
        conc=conc, flux=np.zeros_like(conc),
        concops=np.array(concops, dtype=np.int32),
        concchip=np.array(concchip, dtype=np.float64),
        childops=childops, childchips=childchips,
        compchips=compchips, compops=compops,
        elmnum=np.array(elmnum, dtype=np.int32),
        hnum=np.array(hnum, dtype=np.int32),
        parent_row=parent_row,
        syn_child=syn_child,
        spike_op=spike_op,
        dt=dt, method=model.method, chanmode=model.chanmode, calcmode=model.calcmode,
    )


def _child_pos(row_children, orig_pos):
    for p, _ in row_children:
        if p == orig_pos:
            return p
    raise ValueError("child %d not found" % orig_pos)


# --------------------------------------------------------------------------
# SETUP of many hsolves on every host core
# --------------------------------------------------------------------------
_SENT_TABLES = set()      # in a worker: table keys already returned to the parent
_TABLE_KEYS = {}          # in a worker: id(tablist) -> content key


def _table_key(a: HsolveArrays):
    import hashlib
    k = _TABLE_KEYS.get(id(a.tablist))
    if k is None:
        h = hashlib.blake2b(digest_size=16)
        h.update(struct.pack("<iiidddd", a.ncols, a.xdivs, a.ydivs, a.xmin, a.invdx, a.ymin, a.invdy))
        for arr in (a.tablist, a.xvals, a.yvals):
            h.update(np.ascontiguousarray(arr, dtype=np.float64).tobytes())
        k = h.hexdigest()
        _TABLE_KEYS[id(a.tablist)] = k     # the tables stay alive in _TABLE_CACHE
    return k


def _build_chunk(args):
    """Worker: builds one chunk -- a list of models, or the models
    ``factory(n, start=a, stop=b, **kw)`` generates -- and returns the arrays
    without their tables plus the tables this worker has not returned
    before."""
    what, exact = args
    if isinstance(what, list):
        models = what
    else:
        factory, n, kw, a, b = what
        models = factory(n, start=a, stop=b, **kw)
    out, new = [], {}
    for m in models:
        a = build(m, exact)
        key = None
        if a.ncols:
            key = _table_key(a)
            if key not in _SENT_TABLES:
                _SENT_TABLES.add(key)
                new[key] = (a.tablist, a.xvals, a.yvals)
            a.tablist = a.xvals = a.yvals = None
        out.append((a, key))
    return out, new


def setup_workers(workers: Optional[int] = None) -> int:
    """Processes build_many / build_generated use: ``workers``, else every
    host core this process may run on."""
    import os
    if workers is not None:
        return workers
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def _run_chunks(chunks, workers):
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    tables, out = {}, []
    with ProcessPoolExecutor(min(workers, len(chunks)), mp_context=mp.get_context("spawn")) as pool:
        # results arrive in chunk order, and a worker's chunks in increasing
        # order, so a table is received before any solver that refers to it
        for arrs, new in pool.map(_build_chunk, chunks):
            for k, v in new.items():
                tables.setdefault(k, v)
            for a, key in arrs:
                if key is not None:
                    a.tablist, a.xvals, a.yvals = tables[key]
                out.append(a)
    return out


def build_many(models, exact: bool = False, workers: Optional[int] = None, chunk: int = 2048):
    """``build`` of every model, in order, on ``workers`` processes (default:
    every host core). The reference sets up each hsolve on its own at RESET
    (h_hh_chip_init, do_hget_children, h_funcs_init: hines_chip_init.c:465-
    1260, hines_child.c:81-1549, hines_init.c:361-1273), one after another;
    hsolves are independent, so they are set up here in chunks on a pool of
    spawned processes. Solvers whose composite tables are equal share one
    copy of them, as ``build`` does within one process. The arrays equal
    ``build``'s exactly."""
    models = list(models)
    workers = setup_workers(workers)
    if workers <= 1 or len(models) <= chunk:
        return [build(m, exact) for m in models]
    return _run_chunks([(models[i:i + chunk], exact) for i in range(0, len(models), chunk)], workers)


def build_generated(factory, n: int, exact: bool = False, workers: Optional[int] = None, chunk: int = 512,
                    **kw):
    """``build_many(factory(n, **kw))`` for a generator whose models [a, b)
    come from ``factory(n, start=a, stop=b, **kw)`` alone (configs.random_trees):
    each worker generates its own chunks, so the models never cross a process
    boundary, only the built arrays."""
    workers = setup_workers(workers)
    if workers <= 1 or n <= chunk:
        return [build(m, exact) for m in factory(n, **kw)]
    return _run_chunks([((factory, n, kw, a, min(a + chunk, n)), exact) for a in range(0, n, chunk)], workers)
