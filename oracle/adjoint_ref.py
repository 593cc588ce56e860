"""CPU reference gradient for the engine's differentiated form.

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the engine package.

The reference computes no gradients. This module restates its chanmode 4/5
PROCESS step for the program subset the engine differentiates -- compartments
(COMPT/FCOMPT/LCOMPT), NEWVOLT, CHAN_EK, CHAN, IPOL1V gates with a nonzero
power and ADD_CURR (genesis/src/hines/hines_chip.c:157-600, as restated in
oracle/hsolve_oracle.c orc_chip_update), then the funcs[] elimination walk
(genesis/src/hines/hines_solve.c:140-296, orc_solve) -- on 0-dim torch
float64 tensors on the CPU, and differentiates

    loss = sum_n sum_j (vm[row_j] after step n+1 - trace[n][j])^2

with torch autograd. It walks ops[]/chip[]/funcs[]/ravals[] directly (not the
engine's decoded programs), so it is an independent check of the engine's
hand-written adjoint kernels. Table rows are selected from the float value of
Vm with the reference's bracket cache; the interpolation fraction carries the
derivative. Speed: a few ten thousand compartment-steps per second, so small
cases only.
"""
from __future__ import annotations

import numpy as np
import torch

COMPT, FCOMPT, LCOMPT = 100, 101, 102
CHAN, CHAN_EK, ADD_CURR, IPOL1V, NEWVOLT = 3000, 3001, 3200, 4001, 5100
F_ELIM, F_SET_DIAG, F_SKIP_DIAG, F_CALC = 0, 1, 2, 6


class _Cursor:
    def __init__(self, h):
        if h.ncols:
            self.lo = self.hi = 0.0
        else:
            self.lo, self.hi = -1e20, 1e20
        self.row = 0
        self.base = 0
        self.frac = None   # tensor or float 0


def _val(x):
    return float(x.detach()) if torch.is_tensor(x) else float(x)


def _locate(cur, V, h, interp):
    v = _val(V)
    if interp:
        f = (V - h.xmin) * h.invdx
        if cur.lo > v or v >= cur.hi:
            fv = _val(f)
            if fv < 0.0:
                f = 0.0
            elif fv > h.xdivs:
                f = float(h.xdivs)
            cur.row = int(f)
            f = f - float(cur.row)
            cur.lo = float(h.xvals[cur.row])
            cur.hi = float(h.xvals[cur.row + 1])
            cur.base = cur.row * h.ncols
        else:
            f = f - float(cur.row)
        cur.frac = f
    else:
        if cur.lo > v or v >= cur.hi:
            k = int((v - h.xmin) * h.invdx)
            k = 0 if k < 0 else (h.xdivs if k > h.xdivs else k)
            cur.row = k
            cur.lo = float(h.xvals[k])
            cur.hi = float(h.xvals[k + 1])
            cur.base = k * h.ncols
        cur.frac = 0.0


def _power(g, x, p):
    for _ in range(p):
        g = g * x
    return g


def _step(h, chip, vm, rav, interp, crank):
    ops = h.ops
    tab = h.tablist
    ncols = h.ncols
    n = h.ncompts
    res = [None] * (2 * n)
    cur = _Cursor(h)
    o = c = row = 0
    Ek = Gk = 0.0
    while int(ops[o]) != LCOMPT:
        if int(ops[o]) not in (COMPT, FCOMPT):
            raise ValueError("ops[%d] = %d is not a compartment sentinel" % (o, ops[o]))
        o += 1
        Vm = vm[row]
        sumg = 0.0
        ichan = chip[c] + chip[c + 1]
        c += 2
        while int(ops[o]) > LCOMPT:
            code = int(ops[o])
            o += 1
            if code == NEWVOLT:
                _locate(cur, Vm, h, interp)
                continue
            if code == CHAN_EK:
                Ek = chip[c]
                Gk = chip[c + 1]
                c += 2
            elif code == CHAN:
                Gk = chip[c]
                c += 1
            else:
                raise ValueError("opcode %d is outside the differentiated subset" % code)
            while True:
                k = int(ops[o])
                o += 1
                if k == IPOL1V:
                    b = cur.base + int(ops[o])
                    o += 1
                    if interp:
                        X = tab[b] + cur.frac * (tab[b + ncols] - tab[b])
                        Y = tab[b + 1] + cur.frac * (tab[b + 1 + ncols] - tab[b + 1])
                    else:
                        X, Y = float(tab[b]), float(tab[b + 1])
                    p = int(ops[o])
                    o += 1
                    if p > 0:
                        x = (chip[c] * (2.0 - X) + Y) / X
                    elif p < 0:
                        x = Y / X
                        p = -p
                    else:
                        raise ValueError("tabcurrent gates are outside the differentiated subset")
                    chip[c] = x
                    c += 1
                    Gk = _power(Gk, x, p)
                elif k == ADD_CURR:
                    sumg = sumg + Gk
                    ichan = ichan + Ek * Gk
                    break
                else:
                    raise ValueError("opcode %d is outside the differentiated subset" % k)
        res[2 * row] = Vm + ichan * chip[c]
        res[2 * row + 1] = sumg * chip[c] + chip[c + 1]
        c += 2
        row += 1
    # ---- funcs walk (orc_solve) ----
    f = h.funcs
    fi = ri = 0
    op = int(f[fi]); fi += 1
    if n == 1:
        x = res[0] / res[1]
        vm[0] = x + x - vm[0] if crank else x
        return
    cr = 2
    rv, dv = res[cr], res[cr + 1]
    temp = None
    while True:
        if op == F_ELIM:
            kid = int(f[fi])
            temp = rav[ri] / res[kid + 1]
            ri += 1
            dv = dv - rav[ri] * temp
            ri += 1
            rv = rv - res[kid] * temp
            fi += 1
        elif op == F_SET_DIAG:
            res[cr], res[cr + 1] = rv, dv
            cr += 2
            rv, dv = res[cr], res[cr + 1]
        elif op == F_SKIP_DIAG:
            res[cr], res[cr + 1] = rv, dv
            cr += 4
            rv, dv = res[cr], res[cr + 1]
        elif op in (3, 4, 5):
            raise ValueError("symmetric-compartment funcs are outside the differentiated subset")
        else:
            break
        op = int(f[fi]); fi += 1
    vrow = n - 1
    rv = rv / dv
    vm[vrow] = rv + rv - vm[vrow] if crank else rv
    res[cr] = rv
    cr -= 2
    rv = res[cr]
    while True:
        op = int(f[fi]); fi += 1
        if op == F_ELIM:
            rv = rv - rav[ri] * res[int(f[fi])]
            ri += 1
            fi += 1
        elif op == F_CALC:
            rv = rv / res[cr + 1]
            vrow -= 1
            vm[vrow] = rv + rv - vm[vrow] if crank else rv
            res[cr] = rv
            cr -= 2
            if cr >= 0:
                rv = res[cr]
        else:
            break


def loss_and_gradient(h, nsteps, rows, trace):
    """Loss and its gradient with respect to h.chip, h.ravals and h.vm (numpy
    arrays of the same shapes). ``rows``: target rows; ``trace``:
    [nsteps][len(rows)] target Vm after each step."""
    trace = np.asarray(trace, dtype=np.float64).reshape(nsteps, len(rows))
    chip_t = torch.tensor(np.asarray(h.chip, dtype=np.float64), requires_grad=True)
    rav_t = torch.tensor(np.asarray(h.ravals, dtype=np.float64), requires_grad=True)
    vm_t = torch.tensor(np.asarray(h.vm, dtype=np.float64), requires_grad=True)
    chip = list(chip_t.unbind())
    rav = list(rav_t.unbind()) if len(h.ravals) else []
    vm = list(vm_t.unbind())
    interp = h.calcmode != 0
    crank = h.method == 11
    loss = torch.zeros((), dtype=torch.float64)
    for n in range(nsteps):
        _step(h, chip, vm, rav, interp, crank)
        for j, r in enumerate(rows):
            d = vm[r] - float(trace[n, j])
            loss = loss + d * d
    loss.backward()
    z = lambda t, like: (t.grad.numpy().copy() if t.grad is not None else np.zeros(len(like)))
    return float(loss.detach()), z(chip_t, h.chip), z(rav_t, h.ravals), z(vm_t, h.vm)
