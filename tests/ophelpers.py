"""Hand-assembled hsolve programs for opcode coverage tests.

Builds the flat arrays (ops[], chip[], givals[], tables, conc ...) of small
hsolves directly, for opcodes and table kinds the benchmark models do not
produce: GHK, Nernst, tabcurrent and TABGHK gates, instantaneous gates,
powers 5 and 6, 2-D tables, DOMAIN, ELMMPUMP, Mg block, SYN3, chanmode 5.
Opcode values follow genesis/src/hines/hines_defs.h:178-222.
"""
from types import SimpleNamespace

import numpy as np

(COMPT, FCOMPT, LCOMPT, SPIKE, ELMMPUMP, CONC_VAL, NERNST, GHK, CHAN, CHAN_EK, SAME_GHK, DO_TABGHK,
 ADD_CURR, FLUX, SCALE_FLUX, STORE_ALLI, IPOL1V, IPOL1C, IPOL2V, IPOL2C, SYN2, SYN3, MGBLOCK, NEWVOLT,
 NEWCONC1, NEWCONC2, DOMAIN) = (100, 101, 102, 200, 500, 1000, 2000, 2010, 3000, 3001, 3002, 3003, 3200,
                                3300, 3301, 3501, 4001, 4002, 4003, 4004, 4100, 4101, 4200, 5100, 5110,
                                5111, 5112)
CACONC, LCACONC = 10200, 10202
# concops (hines_defs.h:210-222)
CONC, FCONC, LCONC, FLUXCONC = 10100, 10101, 10102, 10103
TAUPUMP, CTAUPUMP, MMPUMP, HILLPUMP, PHILLPUMP, BUFFER, POOL = 11000, 11001, 11010, 11011, 11012, 12000, 12100


class Compt:
    """One compartment's op stream. Items are ints (ops[] words) or floats
    wrapped by chip() (chip[] values consumed in stream order)."""

    def __init__(self, emrm, inject, tbyc, diag, rm, vm0):
        self.emrm, self.inject, self.tbyc, self.diag, self.rm, self.vm0 = emrm, inject, tbyc, diag, rm, vm0
        self.ops, self.chip = [], []
        self.ngiv = 0

    def op(self, *words, chips=(), giv=0):
        self.ops += list(words)
        self.chip += list(chips)
        self.ngiv += giv
        return self


def tables(ncols, xdivs, xmin=-0.1, xmax=0.05, seed=0, ydivs=0, ymin=0.0, ymax=1.0):
    """Random smooth tables shaped like the trapezoid-transformed gate tables
    hsolve builds: even columns B' = 1 + dt/2*B >= 1, odd columns A' >= 0."""
    rng = np.random.default_rng(seed)
    rows = xdivs + 1
    x = np.linspace(0, 1, rows)[:, None]
    base = 1.0 + 0.05 * rng.random((1, ncols)) + 0.05 * (1 + np.sin(3 * x + rng.random((1, ncols)) * 6))
    tab = base.copy()
    tab[:, 1::2] = 0.4 * base[:, 1::2] * (0.5 + 0.5 * np.cos(2 * x + rng.random((1, ncols // 2)) * 6))
    dx = (xmax - xmin) / xdivs
    xv, v = [], xmin
    for _ in range(rows):
        xv.append(v)
        v += dx
    xv.append(xv[-1])
    out = dict(ncols=ncols, xdivs=xdivs, xmin=xmin, invdx=1.0 / dx,
               tablist=np.concatenate([tab.ravel(), tab[-1]]), xvals=np.array(xv))
    if ydivs:
        dy = (ymax - ymin) / ydivs
        yv, v = [], ymin
        for _ in range(ydivs + 1):
            yv.append(v)
            v += dy
        yv.append(yv[-1])
        out.update(ydivs=ydivs, ymin=ymin, invdy=1.0 / dy, yvals=np.array(yv))
    else:
        out.update(ydivs=0, ymin=0.0, invdy=0.0, yvals=np.zeros(0))
    return out


def solver(compts, tabs, dt=2e-5, conc=(), stablist=(), concops=(), concchip=(), chanmode=4, calcmode=1,
           crank=False, parents=None, diff=None):
    """Arrays of one hsolve. parents: Hines-order parent rows (None = every
    compartment its own root), used to emit funcs[]/ravals[]. diff: the
    diffusion-system arrays (dconc, nshells, nshrows, nshfix, fbufval,
    covals0, bufvals) of do_h_conc_solve, or None."""
    n = len(compts)
    ops, chip, giv, vm = [], [], [0.0], []
    for i, c in enumerate(compts):
        ops.append(FCOMPT if i == 0 else COMPT)
        ops += c.ops
        chip += [c.emrm, c.inject] + c.chip + [c.tbyc, c.diag]
        giv += [c.rm, 0.0] + [0.0] * c.ngiv + [0.0]
        vm.append(c.vm0)
    ops.append(LCOMPT)
    funcs, ravals = _funcs(n, parents)
    return SimpleNamespace(
        ncompts=n, ops=np.array(ops, np.int32), chip=np.array(chip, np.float64),
        funcs=np.array(funcs, np.int32), ravals=np.array(ravals, np.float64), vm=np.array(vm, np.float64),
        givals=np.array(giv, np.float64), stablist=np.array(stablist, np.float64),
        conc=np.array(conc, np.float64), concops=np.array(concops, np.int32),
        concchip=np.array(concchip, np.float64), childops=np.zeros(1, np.int32),
        childchips=np.zeros(1, np.int32), dt=dt, method=11 if crank else 10, crank=1 if crank else 0,
        chanmode=chanmode, calcmode=calcmode, diff=diff, **tabs)


def _funcs(n, parents):
    """funcs[] of asymmetric compartments (the h_funcs_init emission rules,
    genesis/src/hines/hines_init.c:561-1212) with arbitrary coefficients."""
    if parents is None:
        parents = [-1] * n
    kids = [[] for _ in range(n)]
    for r, p in enumerate(parents):
        if p >= 0:
            kids[p].append(r)
    funcs, ravals = [], []
    skip = False
    for i in range(n):
        if skip:
            skip = False
        elif kids[i] or parents[i] == -1:
            if i > 1:
                funcs.append(1)
        elif i > 1:
            funcs.append(2)
            skip = True
        for k in sorted(kids[i]):
            funcs += [0, 2 * k]
            ravals += [-0.011 * (k + 1), -0.013 * (i + 1)]
    funcs.append(7)
    for i in range(n - 2, -1, -1):
        if parents[i] != -1:
            funcs += [0, 2 * parents[i]]
            ravals.append(-0.012 * (i + 1))
        funcs.append(6)
    funcs.append(7)
    return funcs, ravals


def diffusion_system(rng, nshells, nfix=0, ndif=0, dt=2e-5, crank=True):
    """covals0 / bufvals of one difshell system with nfix fixed and ndif
    diffusible buffers per shell, in the order h_setup_conc_solve
    (genesis/src/hines/hines_conc_init.c:313-475) emits them: per shell, per
    row (fixed buffers, diffusible buffers, the shell): fixed buffer
    dt*kBb*Btot; diffusible rows the down- and up-coupling
    2*dt2*D*surf/(vol*(thick+thick')) (one of them at the first and last
    shell). Shell geometry and rate constants are drawn from plausible
    ranges (thickness 0.1-0.5 um, D 2e-10 m^2/s for Ca, kBf 1e5-1e6
    /(mM s), kBb 50-500 /s, Btot 0.01-0.2 mM)."""
    dt2 = dt / 2.0 if crank else dt
    w = nfix + ndif + 1
    thick = rng.uniform(0.1e-6, 0.5e-6, nshells)
    vol = rng.uniform(0.5, 2.0, nshells) * thick * 1e-10
    surf = rng.uniform(0.8, 1.2, nshells + 1) * 1e-10
    Dca, Dbuf = 2e-10, rng.uniform(2e-11, 8e-11, ndif)
    kf, kb, btot = (rng.uniform(1e5, 1e6, nfix + ndif), rng.uniform(50, 500, nfix + ndif),
                    rng.uniform(0.01, 0.2, nfix + ndif))
    bufvals = []
    for b in range(nfix + ndif):
        bufvals += [dt2 * kf[b], dt2 * kb[b], dt * kb[b] * btot[b]]
    cov0 = []
    for m in range(nshells):
        for r in range(w):
            if r < nfix:
                cov0.append(dt * kb[r] * btot[r] * rng.uniform(0.9, 1.1))
                continue
            D = Dbuf[r - nfix] if r < w - 1 else Dca
            diffc = 2.0 * dt2 * D / vol[m]
            t0 = 2 * thick[0] if m == 1 else thick[m - 1] if m else 0.0
            if m < nshells - 1:
                if m:
                    cov0.append(diffc * surf[m] / (t0 + thick[m]))
                    cov0.append(diffc * surf[m + 1] / (thick[m] + thick[m + 1]))
                else:
                    cov0.append(diffc * surf[1] / (2 * thick[0] + thick[1]))
            else:
                cov0.append(diffc * surf[m] / (thick[m - 1] + thick[m]))
    # equilibrium-ish initial concentrations: free buffer, then Ca 50-100 nM
    conc = []
    for m in range(nshells):
        ca = rng.uniform(5e-5, 1e-4)
        conc += [btot[b] * kb[b] / (kb[b] + kf[b] * ca) for b in range(nfix + ndif)] + [ca]
    return np.array(cov0), np.array(bufvals), conc
