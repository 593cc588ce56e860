"""Generates the reference-run fixtures under tests/golden/:

* ref_trajectories.npz: small hsolve models (arrays as the SETUP
  restatement builds them) and their state after N steps of the reference's
  OWN step code (genesis/src/hines/hines_4chip.c, hines_4nichip.c,
  hines_solve.c, hines_conc_4chip.c compiled from the reference sources by
  oracle/Makefile into oracle/_ref/libhsolve_ref.so);
* ref_opcodes.npz: every hand-assembled opcode program of tests/opprograms.py
  in each of its three step modes (chanmode 4, chanmode 5 under
  Crank-Nicolson, calcmode 0), with its state (vm, chip, conc, givals, ops)
  after NSTEPS steps of the same reference code, and a digest of its input
  arrays so that a test notices when a program is no longer the one the
  fixture was made from.

Run in a container that has the reference sources:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "genesis-2.4_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

import pyoracle  # noqa: E402
from gbhsolve import configs, model  # noqa: E402

CASES = [
    ("ap_verify_8x210", lambda: model.build(configs.ap_verify(8)), 210),
    ("cables6_crank", lambda: model.build(configs.cables(6, gk_dend=36.0, method=model.CRANK)[0]), 200),
    ("cables6_euler_calc0", lambda: _calc0(model.build(configs.cables(6, gk_dend=36.0)[0])), 200),
    ("tree40_ca", lambda: model.build(configs.random_trees(1, size_range=(40, 40), seed=3)[0]), 300),
]


def _calc0(h):
    h.calcmode = 0
    return h


def opcode_fixtures():
    import opprograms as P
    out = {"tags": [], "nsteps": np.array(P.NSTEPS)}
    for name in sorted(P.PROGRAMS):
        for mode in P.MODES:
            h, libm = P.build(name, *mode)
            tag = P.mode_tag(name, *mode)
            s = pyoracle.Solver(h)
            s.run(P.NSTEPS, "reference")
            out["tags"].append(tag)
            out[tag + "/digest"] = np.array(P.input_digest(h))
            out[tag + "/libm"] = np.array(bool(libm))
            P.to_fixture(h, tag, out)
            for k in ("vm", "chip", "givals", "ops"):
                out[tag + "/" + k] = getattr(s, k).copy()
            out[tag + "/conc"] = s.conc[:len(h.conc)].copy()
            print(tag, "vm[0] = %.12g" % s.vm[0])
    out["tags"] = np.array(out["tags"])
    np.savez_compressed(os.path.join(HERE, "ref_opcodes.npz"), **out)


def main():
    pyoracle.ensure_built(with_reference=True)
    opcode_fixtures()
    out = {"names": np.array([c[0] for c in CASES])}
    for name, make, nsteps in CASES:
        h = make()
        s = pyoracle.Solver(h)
        s.run(nsteps, "reference")
        for k in ("ops", "chip", "funcs", "ravals", "vm", "givals", "tablist", "xvals", "yvals", "stablist",
                  "conc", "concops", "concchip", "childops", "childchips"):
            out[name + "/" + k] = np.asarray(getattr(h, k))
        out[name + "/scalars"] = np.array([h.ncompts, h.ncols, h.xdivs, h.xmin, h.invdx, h.ydivs, h.ymin, h.invdy,
                                           h.dt, h.crank, h.chanmode, h.calcmode], dtype=np.float64)
        out[name + "/nsteps"] = np.array(nsteps)
        out[name + "/vm_ref"] = s.vm.copy()
        out[name + "/chip_ref"] = s.chip.copy()
        print(name, "vm[-1] = %.12g" % s.vm[-1])
    np.savez_compressed(os.path.join(HERE, "ref_trajectories.npz"), **out)


if __name__ == "__main__":
    main()
