"""Generates tests/golden/symcompt.npz: hsolve models of branched cells made
of SYMMETRIC compartments, with the elimination program the reference's own
SETUP emits for them and their state after N steps of the reference's own
step code.

* funcs[], ravals[] and the constant diagonal terms come from the reference's
  h_funcs_init / do_hnum (genesis/src/hines/hines_init.c:317-1273, symflag 1)
  compiled from the reference sources into oracle/_ref/libhsetup_ref.so
  (oracle/ref_setup.c). Symmetric compartments couple the children of a
  branch point with each other, so the program carries COPY_ARRAY,
  FASTSIBARRAY_ELIM and SIBARRAY_ELIM tokens and rewrites part of ravals[]
  every step.
* The rest of each model (ops[], chip[], tables, pools) is what
  gbhsolve.model builds for the same cell; chip[]'s diagonal terms are
  replaced by the reference's symmetric ones.
* shared/tablist, xvals, yvals: the channel tables of the HH cases; a case
  with another channel mix carries its own (<case>/tablist ...).
* vm_ref/chip_ref: after `nsteps` steps of do_chip_hh4_update +
  do_h4_conc_chip_update + do_euler_hsolve/do_crank_hsolve (oracle/_ref/
  libhsolve_ref.so).
* asym_*: the reference setup's program for the same cells as asymmetric
  compartments, which gbhsolve.model's restatement must reproduce exactly.

Run in a container that has the reference sources:
    python tests/golden/make_symcompt.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "genesis-2.4_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import pyoracle  # noqa: E402
from gbhsolve import configs, model  # noqa: E402

SETUP_LIB = os.path.join(REPO, "oracle", "_ref", "libhsetup_ref.so")


_HH = []


def branched_cell(parents, seed, inject=0.3e-9, gk_dend=36.0, dend_len=20e-6, dia_range=(0.5e-6, 3e-6),
                  with_ca=False):
    """Soma (HH Na/K; with_ca: a Ca channel feeding a Ca_concen pool and a
    Ca-dependent K channel) plus dendrites on the given parent list, dendritic
    K channel on every dendrite; diameters seeded. Every cell shares the same
    channel types (one set of tables per channel mix)."""
    rng = np.random.default_rng(seed)
    if not _HH:
        _HH.extend(configs.hh_channels(-0.065))
        _HH.extend(configs.ca_channels())
    na, k, ca, kca = _HH
    sli, PI = configs.sli, configs.PI
    sl, sd = 30e-6, 30e-6
    sa, sx = sl * PI * sd, PI * (sd / 2) ** 2
    s = model.Compartment(Em=sli(-0.065), Rm=sli(0.33 / sa), Cm=sli(0.01 * sa), Ra=sli(0.3 * sl / sx),
                          initVm=sli(-0.065), inject=sli(inject), parent=parents[0])
    s.children = [model.TabChannel(na, Gbar=sli(1200.0 * sa)), model.TabChannel(k, Gbar=sli(360.0 * sa))]
    if with_ca:
        B = 1.0 / (2 * 96485.3415 * sa * 0.1e-6)
        s.children += [model.TabChannel(ca, Gbar=sli(40.0 * sa), flux_to=4),
                       model.TabChannel(kca, Gbar=sli(100.0 * sa), conc_src=4),
                       model.CaConcen(tau=0.02, B=B, Ca_base=5e-5, thick=0.1e-6)]
    out = [s]
    for c in range(1, len(parents)):
        dd = float(rng.uniform(*dia_range))
        da, dx = dend_len * PI * dd, PI * (dd / 2) ** 2
        d = model.Compartment(Em=sli(-0.065), Rm=sli(0.33 / da), Cm=sli(0.01 * da), Ra=sli(0.3 * dend_len / dx),
                              initVm=sli(-0.065), parent=parents[c])
        if gk_dend:
            d.children = [model.TabChannel(k, Gbar=sli(gk_dend * da))]
        out.append(d)
    return out


def star(nbranch, length):
    """Soma with `nbranch` unbranched dendrites of `length` compartments."""
    parents = [-1]
    for _ in range(nbranch):
        prev = 0
        for _ in range(length):
            parents.append(prev)
            prev = len(parents) - 1
    return parents


def shift(parents, base):
    return [p + base if p >= 0 else -1 for p in parents]


def cases():
    """(name, Model, nsteps) of every fixture case. The reference's symmetric
    SETUP accepts branch points of at most two children: with three or more,
    h_funcs_init stops on its own consistency check ("Bug #8",
    hines_init.c:960-964), so no case has them."""
    out = []
    rng = np.random.default_rng(3)
    t12 = configs.random_binary_tree(rng, 12)
    t30 = configs.random_binary_tree(rng, 30)
    full7 = [-1, 0, 0, 1, 1, 2, 2]
    out.append(("sym_binary12_euler", model.Model(branched_cell(t12, 11), dt=configs.sli(20e-6)), 300))
    out.append(("sym_binary30_crank",
                model.Model(branched_cell(t30, 12), dt=configs.sli(20e-6), method=model.CRANK), 300))
    out.append(("sym_star2x3_euler", model.Model(branched_cell(star(2, 3), 13), dt=configs.sli(20e-6)), 300))
    out.append(("sym_full7_crank",
                model.Model(branched_cell(full7, 14), dt=configs.sli(20e-6), method=model.CRANK), 300))
    two = branched_cell(t12, 15) + branched_cell(shift(star(2, 2), 12), 16, inject=0.5e-9)
    out.append(("sym_two_trees_euler", model.Model(two, dt=configs.sli(20e-6)), 300))
    t48 = configs.random_binary_tree(rng, 48)   # above the engine's one-neuron-per-warp threshold
    out.append(("sym_binary48_euler", model.Model(branched_cell(t48, 17, inject=0.6e-9), dt=configs.sli(20e-6)), 300))
    t20 = configs.random_binary_tree(rng, 20)
    out.append(("sym_binary20_ca_crank", model.Model(branched_cell(t20, 18, inject=0.8e-9, with_ca=True),
                                                     dt=configs.sli(20e-6), method=model.CRANK), 400))
    return out


def ref_setup(m, symflag):
    """hnum, funcs, ravals, diagonal terms from the reference's SETUP."""
    lib = ctypes.CDLL(SETUP_LIB)
    cs = m.compartments
    n = len(cs)
    par = np.array([c.parent for c in cs], np.int32)
    Ra = np.array([c.Ra for c in cs], np.float32)
    Cm = np.array([c.Cm for c in cs], np.float32)
    Rm = np.array([c.Rm for c in cs], np.float32)
    hnum = np.zeros(n, np.int32)
    elm = np.zeros(n, np.int32)
    diag = np.zeros(n)
    nf, nr = ctypes.c_int(0), ctypes.c_int(0)
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    funcs, ravals = np.zeros(1, np.int32), np.zeros(1)
    for _ in range(2):   # first call reports the sizes
        rc = lib.ref_funcs_init(n, ptr(par), ptr(Ra), ptr(Cm), ptr(Rm), int(m.method), ctypes.c_double(m.dt),
                                symflag, ptr(hnum), ptr(elm), ptr(funcs), ctypes.byref(nf), ptr(ravals),
                                ctypes.byref(nr), ptr(diag))
        if rc == 0:
            break
        if rc != -1:
            raise RuntimeError("reference setup failed (%d)" % rc)
        funcs, ravals = np.zeros(nf.value, np.int32), np.zeros(max(nr.value, 1))
    return hnum, funcs, ravals[:nr.value], diag


def symmetric_arrays(m):
    """The model's arrays with the reference's symmetric elimination program."""
    h = model.build(m)
    hnum, funcs, ravals, diag = ref_setup(m, 1)
    assert np.array_equal(hnum, h.hnum)
    n = h.ncompts
    chip = h.chip.copy()
    for i in range(n):
        chip[len(chip) - 1 if i == n - 1 else h.compchips[i + 1] - 1] = diag[i]
    h.chip = chip
    h.funcs = funcs
    h.ravals = ravals
    return h


def main():
    pyoracle.ensure_built(with_reference=True)
    out = {}
    names = []
    for name, m, nsteps in cases():
        h = symmetric_arrays(m)
        s = pyoracle.Solver(h)
        s.run(nsteps, "reference")
        for k in ("ops", "chip", "funcs", "ravals", "vm", "givals", "stablist",
                  "conc", "concops", "concchip", "childops", "childchips"):
            out[name + "/" + k] = np.asarray(getattr(h, k))
        for k in ("tablist", "xvals", "yvals"):   # stored once unless a case's channel mix differs
            if "shared/" + k not in out:
                out["shared/" + k] = np.asarray(getattr(h, k))
            elif not np.array_equal(out["shared/" + k], getattr(h, k)):
                out[name + "/" + k] = np.asarray(getattr(h, k))
        out[name + "/scalars"] = np.array([h.ncompts, h.ncols, h.xdivs, h.xmin, h.invdx, h.ydivs, h.ymin, h.invdy,
                                           h.dt, h.crank, h.chanmode, h.calcmode], dtype=np.float64)
        out[name + "/nsteps"] = np.array(nsteps)
        out[name + "/vm_ref"] = s.vm.copy()
        out[name + "/chip_ref"] = s.chip.copy()
        out[name + "/parents"] = np.array([c.parent for c in m.compartments], np.int32)
        _, af, ar, ad = ref_setup(m, 0)
        out[name + "/asym_funcs"] = af
        out[name + "/asym_ravals"] = ar
        out[name + "/asym_diag"] = ad
        toks = set(int(t) for t in h.funcs)
        print(name, "n=%d nfuncs=%d nravals=%d sym tokens %s vm[-1] = %.12g"
              % (h.ncompts, len(h.funcs), len(h.ravals), sorted(toks & {3, 4, 5}), s.vm[-1]))
        names.append(name)
    out["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "symcompt.npz"), **out)


if __name__ == "__main__":
    main()
