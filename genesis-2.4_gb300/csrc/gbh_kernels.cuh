// gbh_kernels.cuh -- device code of the GB300 hsolve step engine.
//
// One warp owns one tile: 32 neurons (trees) with identical compartment
// programs, one neuron per lane. Per-neuron data is neuron-interleaved
// (row r of lane l at [r*32 + l]) so every warp access is one contiguous
// 256-byte line. A step is
//   1. channel phase: each lane walks its compartments in Hines row order,
//      running the decoded program of every compartment (the reference's
//      do_chip_hh4_update, genesis/src/hines/hines_chip.c:157-600), and
//      leaves (rhs, diag) of each row in the warp's shared-memory columns;
//   2. pool phase: Ca pools (do_h4_conc_chip_update, hines_conc_chip.c:79-219);
//   3. elimination: forward sweep in ascending row order pushing each row's
//      contribution into its parent, root solve, backward substitution in
//      descending order (do_euler_hsolve / do_crank_hsolve, hines_solve.c:
//      140-296), on the lane's private shared-memory columns.
// Arithmetic keeps the reference's operand order; the FP64 build compiles
// with --fmad=false so results match the CPU solver bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include "gbh_internal.h"
#include "gbh_devfn.cuh"

namespace gbh {


// Per-type constants of the compartment interpreter.
template <typename G>
struct ChanEnv {
    const G *tab;
    const double *xvals, *yvals;
    TableGeom tg;
    int ncols;
    bool interp, c5, has_cd;
};

// State the reference carries from one compartment to the next within a
// step (table cursors and their bases, the selected conc, the last channel's
// Ek/Gk/Ik, GHK): reset at the start of every step.
struct ChanState {
    VCursor vc, cc;
    double save_frac;
    int tab_base, ctab_base, sel;
    double Ek, Gk, gmax, Ik, GHK;
    int doGHK;
};

__device__ __forceinline__ void chan_state_reset(ChanState &cs, int ncols)
{
    if (ncols) { cs.vc.lo = cs.vc.hi = 0.0; } else { cs.vc.lo = -1e20; cs.vc.hi = 1e20; }
    cs.vc.row = cs.vc.base = 0;
    cs.vc.frac = 0.0;
    cs.cc.lo = cs.cc.hi = 0.0;
    cs.cc.row = cs.cc.base = 0;
    cs.cc.frac = 0.0;
    cs.save_frac = 0.0;
    cs.tab_base = cs.ctab_base = cs.sel = 0;
    cs.Ek = cs.Gk = cs.gmax = cs.Ik = cs.GHK = 0.0;
    cs.doGHK = 0;
}

// One neuron's rows: parameter fields P, integer state I, conc C, flux F,
// givals G, codiag CD at stride STR (32: lane-interleaved tile, 1: wide
// tile); ring: its synchan event rows (lane-interleaved in both layouts).
struct ChanRows {
    double *P;
    int *I;
    double *C, *F, *G, *CD, *IT;
    unsigned *ring;
    int64_t neuron;
    bool active;
};

// One compartment's program (do_chip_hh4_update's body for one compartment,
// genesis/src/hines/hines_chip.c:157-600): leaves its row's right-hand side
// R and diagonal D. pc advances past the compartment. Returns false on an
// unknown micro-op.
template <typename G, bool GIV, int STR>
__device__ __forceinline__ bool chan_compartment(const DevView &v, const ChanEnv<G> &E, ChanState &cs,
                                                 const ChanRows &N, const int *&pc, double Vm, long long step,
                                                 double &R, double &D)
{
    VCursor &vc = cs.vc, &cc = cs.cc;
    double &save_frac = cs.save_frac;
    int &tab_base = cs.tab_base, &ctab_base = cs.ctab_base, &sel = cs.sel;
    double &Ek = cs.Ek, &Gk = cs.Gk, &gmax = cs.gmax, &Ik = cs.Ik, &GHK = cs.GHK;
    int &doGHK = cs.doGHK;
    const G *tab = E.tab;
    const TableGeom &tg = E.tg;
    const double *xvals = E.xvals, *yvals = E.yvals;
    const int ncols = E.ncols;
    const bool interp = E.interp, c5 = E.c5;
    const int64_t neuron = N.neuron;
    const bool active = N.active;
    (void)neuron;
    (void)active;
    double sumg = 0.0, ichan = 0.0, Im = 0.0;
    for (;;) {

        const int code = pc[0];
        if (code == M_BEGIN) {
            const double emrm = N.P[(pc[1]) * STR];
            ichan = emrm + N.P[(pc[2]) * STR];
            if (GIV) {
                Im = emrm - Vm / N.P[(pc[3]) * STR];
                N.G[(pc[4]) * STR] = Im;
            }
            pc += 5;
        } else if (code == M_NEWVOLT) {
            locate(vc, Vm, tg.xmin, tg.invdx, tg.xdivs, xvals, ncols, interp);
            pc += 1;
        } else if (code == M_CONCVAL) {
            sel = pc[1];
            N.F[(sel) * STR] = 0.0;
            pc += 2;
        } else if (code == M_DOMAIN) {
            const double concen = N.P[(pc[1]) * STR] * Ik;
            locate(cc, concen, tg.ymin, tg.invdy, tg.ydivs, yvals, ncols, interp);
            ctab_base = cc.base;
            pc += 2;
        } else if (code == M_NEWCONC2) {
            const double concen = N.C[(pc[1]) * STR];
            tab_base = ctab_base;
            save_frac = cc.frac;
            locate(cc, concen, tg.ymin, tg.invdy, tg.ydivs, yvals, ncols, interp);
            ctab_base = cc.base;
            pc += 2;
        } else if (code == M_NEWCONC1) {
            const double concen = N.C[(sel) * STR];
            locate(cc, concen, tg.ymin, tg.invdy, tg.ydivs, yvals, ncols, interp);
            ctab_base = cc.base;
            pc += 1;
        } else if (code == M_SPIKE) {
            if (!v.spike_pre)   // else done by k_spikes before the step
                N.I[(pc[2]) * STR] = spike_op(v, Vm, N.P[(pc[1]) * STR], N.I[(pc[2]) * STR], N.I[(pc[3]) * STR],
                                              active, neuron, step);
            pc += 4;
        } else if (code == M_ELMMPUMP) {
            const double cx = N.C[(sel) * STR];
            const double X = 1.0 / (cx + N.P[(pc[1]) * STR]);
            const double vmax = N.P[(pc[2]) * STR];
            ichan += Ik = vmax * cx * X;
            if (GIV) N.G[(pc[4]) * STR] = c5 ? Ik / vmax : Ik;
            Im += Ik;
            if (E.has_cd) N.CD[sel * STR] += N.P[(pc[3]) * STR] * X;   // hines_chip.c:301
            pc += 5;
        } else if (code == M_FLUX) {
            N.F[(sel) * STR] += Ik;
            pc += 1;
        } else if (code == M_SCALE_FLUX) {
            N.F[(sel) * STR] += N.P[(pc[1]) * STR] * Ik;
            pc += 2;
        } else if (code == M_STORE) {
            N.IT[pc[2] * STR] += pc[1] ? Gk : Ik;
            pc += 3;
        } else if (code == M_ITLEAK) {
            N.IT[pc[3] * STR] += N.P[(pc[1]) * STR] - Vm / N.P[(pc[2]) * STR];
            pc += 4;
        } else if (code == M_END) {
            const double tbyc = N.P[(pc[1]) * STR];
            R = Vm + ichan * tbyc;
            D = sumg * tbyc + N.P[(pc[2]) * STR];
            if (GIV) N.G[(pc[3]) * STR] = Im;
            pc += 4;
            break;
        } else {
            // current-producing ops, then the conductance sub-program
            bool current = true;
            if (code == M_GHK) {
                const double cin = N.C[(sel) * STR], cout = N.C[((sel + 1)) * STR];
                GHK = N.P[(pc[1]) * STR];
                double X = Vm * GHK;
                double Y = exp(-X);
                Ek = N.P[(pc[2]) * STR];
                Ik = Ek * (cin - (Y * cout));
                if (fabs(X) < 1.0e-6) {
                    Gk = 1.0 - 0.5 * X;
                    GHK = 0.5 * GHK * Ek * (cin + cout);
                    Ik = -Ik / Gk;
                } else {
                    Gk = 1.0 - Y;
                    GHK = GHK * (Ik / Gk - Ek * GHK * (cin - cout) * Vm * Y / (Gk * Gk));
                    Ik = -X * Ik / Gk;
                }
                Ek = (Ik + GHK * Vm) / GHK;
                gmax = N.P[(pc[3]) * STR];
                Gk = gmax * GHK;
                pc += 4;
            } else if (code == M_SAME_GHK) {
                gmax = N.P[(pc[1]) * STR];
                Gk = gmax * GHK;
                pc += 2;
            } else if (code == M_DO_TABGHK) {
                doGHK = 1;
                pc += 1;
            } else if (code == M_NERNST) {
                Ek = log(N.C[((sel + 1)) * STR] / N.C[(sel) * STR]) * N.P[(pc[1]) * STR];
                gmax = Gk = N.P[(pc[2]) * STR];
                pc += 3;
            } else if (code == M_CHAN) {
                Ek = N.P[(pc[1]) * STR];
                gmax = Gk = N.P[(pc[2]) * STR];
                pc += 3;
            } else if (code == M_CHAN_G) {
                gmax = Gk = N.P[(pc[1]) * STR];
                pc += 2;
            } else {
                current = false;
                if (v.status) atomicOr(v.status, ST_BAD_OP);
                return false;
            }
            if (!current) continue;
            for (;;) {
                const int k = pc[0];
                if (k == M_GATE) {
                    const int kind = pc[1];
                    int b;
                    G X, Y;
                    if (kind == GK_1V || kind == GK_1C) {
                        const VCursor &cu = (kind == GK_1V) ? vc : cc;
                        b = ((kind == GK_1V) ? vc.base : ctab_base) + pc[2];
                        if (interp) {
                            const G fr = (G)cu.frac;
                            X = tab[b];
                            X = X + fr * (tab[b + ncols] - X);
                            Y = tab[b + 1];
                            Y = Y + fr * (tab[b + 1 + ncols] - Y);
                        } else {
                            X = tab[b];
                            Y = tab[b + 1];
                        }
                    } else {
                        const G rf = (G)((kind == GK_2V) ? vc.frac : save_frac);
                        const G cf = (G)cc.frac;
                        b = ((kind == GK_2V) ? vc.base : tab_base) + cc.row + cc.row + pc[2];
                        if (interp) {
                            const int n = b + ncols;
                            X = ((G)1.0 - rf) * (((G)1.0 - cf) * tab[b] + cf * tab[b + 2]) +
                                rf * (((G)1.0 - cf) * tab[n] + cf * tab[n + 2]);
                            Y = ((G)1.0 - rf) * (((G)1.0 - cf) * tab[b + 1] + cf * tab[b + 3]) +
                                rf * (((G)1.0 - cf) * tab[n + 1] + cf * tab[n + 3]);
                        } else {
                            X = tab[b];
                            Y = tab[b + 1];
                        }
                    }
                    tab_base = b + 1;
                    const int p = pc[3];
                    if (p == 0) {
                        Ek = (double)Y;
                        pc += 5;
                        if (doGHK) {
                            GHK = (double)X;
                            doGHK = 0;
                            break;
                        }
                        Gk *= (double)X;   // tabcurrent; M_ADDCURR follows
                        continue;
                    } else {
                        double *st = &N.P[(pc[4]) * STR];
                        G x;
                        int pw = p;
                        if (p > 0) {
                            x = ((G)(*st) * ((G)2.0 - X) + Y) / X;
                        } else {
                            x = Y / X;
                            pw = -p;
                        }
                        *st = (double)x;
                        Gk = (double)gpow<G>((G)Gk, x, pw);
                        pc += 5;
                        continue;
                    }
                } else if (k == M_SYN) {
                    // SYN2_OP / SYN3_OP (hines_chip.c:511-531): decay X, add the
                    // events due now (h_dosynchan, hines_conn.c:62-89), update Y.
                    const double *sl = v.stablist + pc[2];
                    double *px = &N.P[(pc[4]) * STR];
                    double *py = &N.P[(pc[5]) * STR];
                    if (pc[1] >= 0) {
                        const uint64_t key = ((uint64_t)neuron << 24) ^ ((uint64_t)step << 1) ^
                                             (uint64_t)pc[4];
                        if (syn3_uniform(key) <= N.P[(pc[1]) * STR]) *px += sl[3];
                    }
                    double X = *px * sl[0];
                    unsigned *cell = N.ring + ((int64_t)pc[3] * v.ring_len +
                                               (int64_t)(step % v.ring_len)) * LANES;
                    double act;
                    if (syn_due(v, cell, N.P[(pc[6]) * STR], step, act)) X += v.dt * act * sl[3];
                    *px = X;
                    const double Y = X * sl[1] + *py * sl[2];
                    *py = Y;
                    Gk *= Y;
                    pc += 7;
                    continue;
                } else if (k == M_MGBLOCK) {
                    if (GIV) {
                        const int g = pc[4];
                        if (c5) {
                            N.G[(g) * STR] = Gk / gmax;
                            N.G[((g + 1)) * STR] = Gk * (Ek - Vm) / gmax;
                        } else {
                            N.G[(g) * STR] = Gk;
                            N.G[((g + 1)) * STR] = Gk * (Ek - Vm);
                        }
                        N.G[((g + 2)) * STR] = Ek;
                    }
                    const double X = N.P[(pc[1]) * STR] * exp(Vm * N.P[(pc[2]) * STR]);
                    Gk *= X / (X + N.P[(pc[3]) * STR]);
                    pc += 5;
                    continue;
                } else if (k == M_ADDCURR) {
                    // DOADDCURR (hines_chip.c:551-567)
                    const int g = pc[1];
                    sumg += Gk;
                    ichan += Ek * Gk;
                    Ik = Gk * (Ek - Vm);
                    if (GIV) {
                        if (c5) {
                            N.G[(g) * STR] = Gk / gmax;
                            N.G[((g + 1)) * STR] = Ik / gmax;
                        } else {
                            N.G[(g) * STR] = Gk;
                            N.G[((g + 1)) * STR] = Ik;
                        }
                        N.G[((g + 2)) * STR] = Ek;
                    }
                    pc += 2;
                } else {
                    if (v.status) atomicOr(v.status, ST_BAD_OP);
                    return false;
                }
                Im += Ik;
                break;
            }
        }
    }
    return true;
}

// ---------------------------------------------------------------- kernel
// Shared memory per warp: 2 * nslots_max * 32 doubles (diag and rhs columns).
template <typename G, bool GIV>
__global__ void __launch_bounds__(128, 4)
k_steps(DevView v, int tile0, int tile1, int smax, int nsteps, long long step0)
{
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int t = tile0 + blockIdx.x * (blockDim.x >> 5) + wib;
    if (t >= tile1) return;
    const long long sbase = v.step_dev ? *v.step_dev : 0;
    const Tile tl = v.tiles[t];
    const TileType ty = v.types[tl.type];
    const TableGeom tg = v.tgeom[ty.table_set];
    const G *tab = tab_ptr<G>(v, tg.tab_off);
    const double *xvals = v.xyvals + tg.xv_off;
    const double *yvals = tg.yv_off >= 0 ? v.xyvals + tg.yv_off : xvals;
    const int ncols = tg.ncols;
    const bool interp = ty.interp != 0;
    const bool c5 = ty.chanmode5 != 0;
    const bool active = lane < tl.nlanes;

    double *Pw = v.P + tl.fld * LANES + lane;
    int *Iw = v.I + tl.ints * LANES + lane;
    double *Vw = v.V + tl.vm * LANES + lane;
    double *Cw = v.C + tl.pools * LANES + lane;
    double *Gw = v.giv + tl.giv * LANES + lane;
    const int *par = v.parent + tl.topo * LANES + lane;
    const double *Aw = v.A + tl.topo * LANES + lane;
    const double *Bw = v.B + tl.topo * LANES + lane;
    const double *Cbw = v.Cb + tl.topo * LANES + lane;
    double *Dcol = sm + (size_t)wib * 2 * smax * LANES + lane;   // diag column
    double *Rcol = Dcol + (size_t)smax * LANES;                   // rhs column
    const int S = ty.nslots;
    const int64_t neuron = tl.first_neuron + lane;
    double *Fw = v.F + tl.pools * LANES + lane;

    ChanEnv<G> E;
    E.tab = tab;
    E.xvals = xvals;
    E.yvals = yvals;
    E.tg = tg;
    E.ncols = ncols;
    E.interp = interp;
    E.c5 = c5;
    E.has_cd = ty.has_cd != 0;
    ChanRows NR;
    NR.P = Pw;
    NR.I = Iw;
    NR.C = Cw;
    NR.F = Fw;
    NR.G = Gw;
    NR.CD = v.CD ? v.CD + tl.pools * LANES + lane : nullptr;
    NR.IT = v.IT + tl.itot * LANES + lane;
    NR.ring = v.ring + tl.syn * LANES + lane;
    NR.neuron = neuron;
    NR.active = active;

    for (int it = 0; it < nsteps; ++it) {
        const long long step = sbase + step0 + it;
        for (int k = 0; k < ty.nitot; ++k) NR.IT[k * LANES] = 0.0;   // hines_chip.c:134-136
        // ---------------- channel phase ----------------
        ChanState cs;
        chan_state_reset(cs, tg.ncols);
        const int *pc = v.prog + ty.prog_off;
        for (int s = 0; s < S; ++s) {
            double R, D;
            if (!chan_compartment<G, GIV, LANES>(v, E, cs, NR, pc, Vw[s * LANES], step, R, D)) {
                if (v.status) atomicOr(v.status, ST_BAD_OP);
                return;
            }
            Rcol[s * LANES] = R;
            Dcol[s * LANES] = D;
        }

        // ---------------- pool phase ----------------
        {
            PoolLane PL;
            PL.C = Cw;
            PL.F = Fw;
            PL.CR = v.CR ? v.CR + tl.pools * LANES + lane : nullptr;
            PL.CD = v.CD ? v.CD + tl.pools * LANES + lane : nullptr;
            PL.S = v.S ? v.S + tl.scr * LANES + lane : nullptr;
            PL.P = Pw;
            PL.V = Vw;
            PL.dt = v.dt;
            PL.crank = ty.crank;
            if (!pool_phase<LANES>(v.prog + ty.pool_off, PL)) {
                if (v.status) atomicOr(v.status, ST_BAD_OP);
                return;
            }
        }

        // ---------------- elimination ----------------
        if (ty.sym) {
            sym_eliminate<LANES>(v.prog + ty.sym_off, Rcol, Dcol, v.RV + tl.rav * LANES + lane, Vw, ty.crank != 0);
        } else {
        for (int s = 0; s < S; ++s) {
            const int p = par[s * LANES];
            if (p >= 0) {
                const double d = Dcol[s * LANES];
                const double temp = Aw[s * LANES] / d;
                Dcol[p * LANES] -= Bw[s * LANES] * temp;
                Rcol[p * LANES] -= Rcol[s * LANES] * temp;
            }
        }
        for (int s = S - 1; s >= 0; --s) {
            const int p = par[s * LANES];
            double r = Rcol[s * LANES];
            if (p >= 0) r -= Cbw[s * LANES] * Rcol[p * LANES];
            r = r / Dcol[s * LANES];
            Rcol[s * LANES] = r;
            if (ty.crank) {
                const double old = Vw[s * LANES];
                Vw[s * LANES] = r + r - old;
            } else {
                Vw[s * LANES] = r;
            }
        }
        }
        finite_check(v, Vw[0], active);
        // cooperative multi-step launch: every tile's events of this step
        // are in the rings before any tile starts the next step
        if (v.gbar && !grid_sync(v.gbar, gridDim.x, v.status)) return;
    }
}

// ------------------------------------------------------------ stack elimination
// Lane-mapped tiles of large neurons (TileType::stack): one neuron per lane
// as in k_steps, but the rows never sit in shared memory as columns. Each
// neuron's rows are a post-order of its tree (the Hines numbering of
// do_hnum, hines_init.c:317-345: every subtree contiguous, its root last), so
// the forward elimination runs fused with the channel phase, row by row: the
// row's own right-hand side and diagonal, minus its children's contributions
// in ascending row order -- the older children's from a per-lane stack in
// shared memory, the last child's (the previous row) from registers -- and
// then its own contribution, pushed or carried. The pool phase follows (it
// reads Vm and concentrations, never a row's diagonal), then back
// substitution in descending row order from the per-row (rhs, diagonal)
// column in global memory. The operations and their order per row are those
// of the sequential sweep (hines_solve.c:223-296), so FP64 results are the
// reference's bit for bit. Shared memory: cap doubles per lane (16 bytes per
// pending contribution, 8 per pending branch-point solution).
//
// SPLIT: two warps per tile. After a launch's first step the second warp
// runs the channel phase of the rows above the static ones (kSplitRows at
// most; the soma of a tree whose dendrites are passive) and the pool phase,
// leaving each row's (R, D) in shared memory, while the first warp sweeps
// the static rows; the first warp then finishes those rows' forward steps
// and the back substitution. Both warps pass two barriers per step. The
// operations per row are the same either way.
template <typename G, bool GIV, bool SPLIT>
__global__ void __launch_bounds__(SPLIT ? 64 : 32, SPLIT ? 8 : 16)
k_stack(DevView v, int tile0, int tile1, int cap, int nsteps, long long step0)
{
    extern __shared__ double sm[];
    __shared__ int sbad;
    const int lane = threadIdx.x & (LANES - 1);
    const int wid = SPLIT ? (int)(threadIdx.x >> 5) : 0;   // 0 sweeps, 1 computes the channel rows
    const int t = tile0 + blockIdx.x;
    if (t >= tile1) return;
    {
        unsigned dsz;
        asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dsz));
        if (dsz < ((unsigned)cap + (SPLIT ? 2u * kSplitRows : 0u)) * LANES * sizeof(double)) {
            if (v.status && threadIdx.x == 0) atomicOr(v.status, ST_SMEM);
            return;
        }
    }
    if (SPLIT) {
        if (threadIdx.x == 0) sbad = 0;
        __syncthreads();
    }
    const long long sbase = v.step_dev ? *v.step_dev : 0;
    const Tile tl = v.tiles[t];
    const TileType ty = v.types[tl.type];
    const TableGeom tg = v.tgeom[ty.table_set];
    const double *xvals = v.xyvals + tg.xv_off;
    const double *yvals = tg.yv_off >= 0 ? v.xyvals + tg.yv_off : xvals;
    const bool active = lane < tl.nlanes;

    double *Pw = v.P + tl.fld * LANES + lane;
    double *Vw = v.V + tl.vm * LANES + lane;
    double *Cw = v.C + tl.pools * LANES + lane;
    double *Fw = v.F + tl.pools * LANES + lane;
    const int *lt = v.ltop + tl.topo * LANES + lane;
    const double *Aw = v.A + tl.topo * LANES + lane;
    const double *Bw = v.B + tl.topo * LANES + lane;
    const double *Cbw = v.Cb + tl.topo * LANES + lane;
    double2 *col = v.col + tl.topo * LANES + lane;
    double2 *kst = v.kst + tl.topo * LANES + lane;
    double *kri = v.kri + tl.topo * LANES + lane;
    double *stk = sm + lane;      // entry j at stk[j * 32]
    double *rdb = sm + cap * LANES + lane;  // SPLIT: (R, D) of the rows above the static ones
    const int S = ty.nslots;
    const int *pf = v.prog + ty.pf_off;   // per slot: field rows to prefetch; passive rows' fields
    const int nst = GIV ? 0 : ty.nstatic; // static rows (givals off: they would write Im)
    constexpr int kCh = 8;                // rows per chunk
    const bool sp = SPLIT && nst > 0 && S - nst <= kSplitRows;
    // The static rows' kept factors outlive a launch: they are redone (a
    // full first step) only when the fields they come from may have changed
    // since this tile last kept them (a state write bumps *v.sgen); else the
    // first step only refreshes the rhs terms (inputs may set an inject).
    const unsigned sgen = nst > 0 ? *v.sgen : 0u;
    const bool full = nst > 0 && v.tgen[t] != sgen;
    const bool kref = nst > 0 && *v.kref != 0;   // an input writes a static row's rhs fields
    if (SPLIT) __syncthreads();   // both warps read tgen[t] before the sweeping warp rewrites it

    ChanEnv<G> E;
    E.tab = tab_ptr<G>(v, tg.tab_off);
    E.xvals = xvals;
    E.yvals = yvals;
    E.tg = tg;
    E.ncols = tg.ncols;
    E.interp = ty.interp != 0;
    E.c5 = ty.chanmode5 != 0;
    E.has_cd = ty.has_cd != 0;
    ChanRows NR;
    NR.P = Pw;
    NR.I = v.I + tl.ints * LANES + lane;
    NR.C = Cw;
    NR.F = Fw;
    NR.G = v.giv + tl.giv * LANES + lane;
    NR.CD = v.CD ? v.CD + tl.pools * LANES + lane : nullptr;
    NR.IT = v.IT + tl.itot * LANES + lane;
    NR.ring = v.ring + tl.syn * LANES + lane;
    NR.neuron = tl.first_neuron + lane;
    NR.active = active;

    for (int it = 0; it < nsteps; ++it) {
        const long long step = sbase + step0 + it;
        // after a launch's first step the static rows' (rhs term, coupling
        // factor) are in kst: their diagonals do not change within a launch
        // (nothing but channels changes a diagonal; inputs and state writes
        // come between launches), so they skip the diagonal's elimination
        const bool fast = it > 0 || !full;
        const bool refresh = it == 0 && kref;   // (fast) the rhs terms from the fields
        const bool split = sp && fast;
        bool bad = false;
        if (SPLIT && wid == 1 && !split) goto step_end;   // the second warp works in split steps only
        if (!split || wid == 1)
            for (int k = 0; k < ty.nitot; ++k) NR.IT[k * LANES] = 0.0;   // hines_chip.c:134-136
        if (SPLIT && wid == 1) {
            // the rows above the static ones: channel phase into shared
            // memory, then the pool phase (it reads Vm, fluxes and
            // concentrations, never a row of the elimination)
            ChanState cs1;
            chan_state_reset(cs1, tg.ncols);
            const int *pc1 = v.prog + ty.prog_off + 9 * nst;   // a passive row's program is 9 ints
            for (int s = nst; s < S && !bad; ++s) {
                double R, D;
                if (!chan_compartment<G, GIV, LANES>(v, E, cs1, NR, pc1, Vw[s * LANES], step, R, D)) {
                    bad = true;
                } else {
                    rdb[(2 * (s - nst)) * LANES] = R;
                    rdb[(2 * (s - nst) + 1) * LANES] = D;
                }
            }
            if (!bad) {
                PoolLane PL;
                PL.C = Cw;
                PL.F = Fw;
                PL.CR = v.CR ? v.CR + tl.pools * LANES + lane : nullptr;
                PL.CD = NR.CD;
                PL.S = v.S ? v.S + tl.scr * LANES + lane : nullptr;
                PL.P = Pw;
                PL.V = Vw;
                PL.dt = v.dt;
                PL.crank = ty.crank;
                bad = !pool_phase<LANES>(v.prog + ty.pool_off, PL);
            }
            if (bad && v.status) atomicOr(v.status, ST_BAD_OP);
            bar_named(1, 2 * LANES);   // (R, D) ready
            goto step_end;
        }
        {
        const int Send = split ? nst : S;   // the rows this warp sweeps before the barrier
        ChanState cs;
        chan_state_reset(cs, tg.ncols);
        const int *pc = v.prog + ty.prog_off;
        int top = 0;                    // stack entries (two doubles each)
        double cd = 0.0, cr = 0.0;      // contribution carried to the next row
        // the forward step of row s from its own (R, D): children's
        // contributions (stack, then the carried last child) in ascending row
        // order, its (R, D) into the column, its own contribution pushed or
        // carried -- the operations of the sequential sweep (hines_solve.c:247-252).
        // A static row also keeps its rhs term K and its factor a / D.
        auto fwd = [&](int s, double R, double D, int f, double a, double bb, double K) {
            const int np = f & FL_NPOP;
            if (ty.slots) top = ((f >> FL_SLOT_F) & 31) + np;   // the static rows keep no running top
            top -= np;
            for (int j = 0; j < np; ++j) {
                D -= stk[(2 * (top + j)) * LANES];
                R -= stk[(2 * (top + j) + 1) * LANES];
            }
            if (f & FL_CARRY_IN) {
                D -= cd;
                R -= cr;
            }
            col[s * LANES] = make_double2(R, D);
            double temp = 0.0;
            if (f & FL_PARENT) {
                temp = a / D;
                const double pd = bb * temp, pr = R * temp;
                if (f & FL_CARRY_OUT) {
                    cd = pd;
                    cr = pr;
                } else {
                    stk[(2 * top) * LANES] = pd;
                    stk[(2 * top + 1) * LANES] = pr;
                    ++top;
                }
            }
            if (s < nst) {
                kst[s * LANES] = make_double2(K, temp);
                kri[s * LANES] = 1.0 / D;   // IEEE: the correctly rounded reciprocal
            }
        };
        // the same for a static row on later steps: its diagonal and factor
        // are those of the first step, so only the rhs is eliminated (the
        // same operations on R as above); its diagonal contribution bb * temp
        // is formed only for a parent above the static rows
        auto fwd_static = [&](int s, double R, double T, int f) {
            const int np = f & FL_NPOP;
            top -= np;
            for (int j = 0; j < np; ++j) R -= stk[(2 * (top + j) + 1) * LANES];
            if (f & FL_CARRY_IN) R -= cr;
            reinterpret_cast<double *>(col + s * LANES)[0] = R;
            if (f & FL_PARENT) {
                // the diagonal contribution only for a parent above the static
                // rows (a static parent never reads it)
                const double pr = R * T;
                if (f & FL_CARRY_OUT) {
                    cr = pr;
                    if (f & FL_PD) cd = Bw[s * LANES] * T;
                } else {
                    if (f & FL_PD) stk[(2 * top) * LANES] = Bw[s * LANES] * T;
                    stk[(2 * top + 1) * LANES] = pr;
                    ++top;
                }
            }
        };
        // fwd_static for types whose rows pop at most one stacked child: the
        // same operations as selects and predicated stores instead of
        // branches, so consecutive rows' independent work can overlap
        auto fwd_static1 = [&](int s, double R, double T, int f) {
            const bool pop = f & 1;
            top -= pop ? 1 : 0;
            const double sv = stk[(pop ? 2 * top + 1 : 1) * LANES];
            R = pop ? R - sv : R;
            R = (f & FL_CARRY_IN) ? R - cr : R;
            reinterpret_cast<double *>(col + s * LANES)[0] = R;
            const double pr = R * T;
            if (f & FL_PD) {   // a parent above the static rows: its diagonal contribution
                const double pd = Bw[s * LANES] * T;
                if (f & FL_CARRY_OUT) cd = pd;
                else stk[(2 * top) * LANES] = pd;
            }
            cr = (f & FL_CARRY_OUT) ? pr : cr;
            if (f & FL_PUSH) stk[(2 * top + 1) * LANES] = pr;
            top += (f & FL_PUSH) ? 1 : 0;
        };
        // fwd_static1 for TileType::slots: the row's stack entry comes with
        // its flags, so no running top is kept
        auto fwd_static2 = [&](int s, double R, double T, int f) {
            const int sl = (f >> FL_SLOT_F) & 31;
            const double sv = stk[(2 * sl + 1) * LANES];
            R = (f & 1) ? R - sv : R;
            R = (f & FL_CARRY_IN) ? R - cr : R;
            reinterpret_cast<double *>(col + s * LANES)[0] = R;
            const double pr = R * T;
            if (f & FL_PD) {   // a parent above the static rows: its diagonal contribution
                const double pd = Bw[s * LANES] * T;
                if (f & FL_CARRY_OUT) cd = pd;
                else stk[(2 * sl) * LANES] = pd;
            }
            cr = (f & FL_CARRY_OUT) ? pr : cr;
            if (f & FL_PUSH) stk[(2 * sl + 1) * LANES] = pr;
        };
        // a static row on a launch's later step, in the form its type allows
        auto fwd_fast = [&](int s, double R, double T, int f) {
            if (ty.slots) fwd_static2(s, R, T, f);
            else if (ty.np1) fwd_static1(s, R, T, f);
            else fwd_static(s, R, T, f);
        };
        // a static row's rhs term from its fields (as `passive` forms it), kept
        auto kterm = [&](int s) {
            const int *ps = pf + 6 * s;
            const double ichan = Pw[ps[2] * LANES] + Pw[ps[3] * LANES];
            const double K = ichan * Pw[ps[4] * LANES];
            kst[s * LANES].x = K;
            return K;
        };
        // the interpreter's M_BEGIN / M_END arithmetic of a passive row; K
        // is the rhs term ichan * tbyc
        auto passive = [&](int s, const int *ps, double &R, double &D, double &K) {
            const double Vm = Vw[s * LANES];
            const double ichan = Pw[ps[2] * LANES] + Pw[ps[3] * LANES];
            const double tbyc = Pw[ps[4] * LANES];
            const double sumg = 0.0;
            K = ichan * tbyc;
            R = Vm + K;
            D = sumg * tbyc + Pw[ps[5] * LANES];
        };
        // inputs on the static rows' rhs fields: their terms from the fields,
        // once, before the sweep (not inside its chains)
        if (refresh && fast)
            for (int s = 0; s < nst; ++s) kterm(s);
        for (int s0 = 0; s0 < Send && !bad; s0 += kCh) {
            if (fast && s0 + kCh <= nst) {
                double R[kCh], T[kCh];
                int f[kCh];
#pragma unroll
                for (int k = 0; k < kCh; ++k) {
                    const double2 kt = kst[(s0 + k) * LANES];
                    f[k] = lt[(s0 + k) * LANES];
                    R[k] = Vw[(s0 + k) * LANES] + kt.x;
                    T[k] = kt.y;
                }
                if (ty.slots) {
#pragma unroll
                    for (int k = 0; k < kCh; ++k) fwd_static2(s0 + k, R[k], T[k], f[k]);
                } else if (ty.np1) {
#pragma unroll
                    for (int k = 0; k < kCh; ++k) fwd_static1(s0 + k, R[k], T[k], f[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < kCh; ++k) fwd_static(s0 + k, R[k], T[k], f[k]);
                }
                pc += 9 * kCh;
                continue;
            }
            for (int q = s0 + kCh; q < min(s0 + 2 * kCh, Send); ++q) {   // the next chunk's rows, into L1
                for (int f = pf[6 * q]; f <= pf[6 * q + 1]; ++f) prefetch_l1(&Pw[f * LANES]);
                prefetch_l1(&Vw[q * LANES]);
                prefetch_l1(&lt[q * LANES]);
                prefetch_l1(&Aw[q * LANES]);
                prefetch_l1(&Bw[q * LANES]);
            }
            bool all_passive = !GIV && s0 + kCh <= Send;
            for (int k = 0; k < kCh && all_passive; ++k) all_passive = pf[6 * (s0 + k) + 2] >= 0;
            if (all_passive) {
                // every row's own terms first (independent of each other),
                // then the elimination chain through them
                double R[kCh], D[kCh], K[kCh], a[kCh], bb[kCh];
                int f[kCh];
#pragma unroll
                for (int k = 0; k < kCh; ++k) {
                    passive(s0 + k, pf + 6 * (s0 + k), R[k], D[k], K[k]);
                    f[k] = lt[(s0 + k) * LANES];
                    a[k] = Aw[(s0 + k) * LANES];
                    bb[k] = Bw[(s0 + k) * LANES];
                }
#pragma unroll
                for (int k = 0; k < kCh; ++k) {
                    const int s = s0 + k;
                    if (fast && s < nst) {
                        fwd_fast(s, Vw[s * LANES] + kst[s * LANES].x, kst[s * LANES].y, f[k]);
                    } else {
                        fwd(s, R[k], D[k], f[k], a[k], bb[k], K[k]);
                    }
                }
                pc += 9 * kCh;
                continue;
            }
            for (int s = s0; s < min(s0 + kCh, Send) && !bad; ++s) {
                double R, D, K = 0.0;
                const int *ps = pf + 6 * s;
                if (fast && s < nst) {
                    const double2 kt = kst[s * LANES];
                    fwd_fast(s, Vw[s * LANES] + kt.x, kt.y, lt[s * LANES]);
                    pc += 9;
                    continue;
                }
                if (!GIV && ps[2] >= 0) {
                    passive(s, ps, R, D, K);
                    pc += 9;
                } else if (!chan_compartment<G, GIV, LANES>(v, E, cs, NR, pc, Vw[s * LANES], step, R, D)) {
                    if (v.status) atomicOr(v.status, ST_BAD_OP);
                    bad = true;
                    break;
                }
                fwd(s, R, D, lt[s * LANES], Aw[s * LANES], Bw[s * LANES], K);
            }
        }
        if (split) {
            bar_named(1, 2 * LANES);   // the second warp's (R, D) of the rows above the static ones
            for (int s = nst; s < S; ++s)
                fwd(s, rdb[(2 * (s - nst)) * LANES], rdb[(2 * (s - nst) + 1) * LANES], lt[s * LANES],
                    Aw[s * LANES], Bw[s * LANES], 0.0);
        } else if (!bad) {
            PoolLane PL;
            PL.C = Cw;
            PL.F = Fw;
            PL.CR = v.CR ? v.CR + tl.pools * LANES + lane : nullptr;
            PL.CD = NR.CD;
            PL.S = v.S ? v.S + tl.scr * LANES + lane : nullptr;
            PL.P = Pw;
            PL.V = Vw;
            PL.dt = v.dt;
            PL.crank = ty.crank;
            if (!pool_phase<LANES>(v.prog + ty.pool_off, PL)) {
                if (v.status) atomicOr(v.status, ST_BAD_OP);
                bad = true;
            }
        }
        if (!bad) {
        double xn = 0.0;   // solution of the row after
        top = 0;
        // back substitution of row s (hines_solve.c:270-289): its solution
        // from the parent's (the row after, or the branch point on the stack)
        // (selects and predicated stack accesses instead of branches)
        // (TileType::slots: the stack entries come with the flags)
        // A static row divides by its kept D' with the correctly rounded y =
        // 1/D' (kri): q = RN(r y), e = r - D' q (exact, FMA), RN(q + e y) is
        // RN(r / D') (Markstein's theorem: y within half an ulp of 1/D', q
        // within an ulp of r / D'), so the quotient is the division's bits.
        auto bwd = [&](int s, int f, double2 rd, double c, double old, bool stat, double y) {
            const bool xl = f & FL_XLOAD;
            const int rs = ty.slots ? (f >> FL_SLOT_R) & 31 : (xl ? top - 1 : 0);
            const double sv = stk[rs * LANES];
            const double xp = xl ? sv : xn;
            if (!ty.slots) top -= (f & FL_XPOP) ? 1 : 0;
            double r = (f & FL_PARENT) ? rd.x - c * xp : rd.x;
            if (stat) {
                const double q = r * y;
                r = fma(fma(-rd.y, q, r), y, q);
            } else {
                r = r / rd.y;
            }
            if (f & FL_XPUSH) stk[(ty.slots ? (f >> FL_SLOT_W) & 31 : top) * LANES] = r;
            if (!ty.slots) top += (f & FL_XPUSH) ? 1 : 0;
            xn = r;
            Vw[s * LANES] = ty.crank ? r + r - old : r;
        };
        int s1 = S - 1;
        // chunks: every row's loads, then the chain; the rows above the
        // static ones first (IEEE division), then the static rows
        for (; s1 + 1 - nst >= kCh; s1 -= kCh) {
            int f[kCh];
            double2 rd[kCh];
            double c[kCh], old[kCh];
#pragma unroll
            for (int k = 0; k < kCh; ++k) {
                const int s = s1 - k;
                f[k] = lt[s * LANES];
                rd[k] = col[s * LANES];
                c[k] = Cbw[s * LANES];
                old[k] = ty.crank ? Vw[s * LANES] : 0.0;
            }
#pragma unroll
            for (int k = 0; k < kCh; ++k) bwd(s1 - k, f[k], rd[k], c[k], old[k], false, 0.0);
        }
        for (; s1 >= nst; --s1)
            bwd(s1, lt[s1 * LANES], col[s1 * LANES], Cbw[s1 * LANES], ty.crank ? Vw[s1 * LANES] : 0.0, false, 0.0);
        for (; s1 + 1 >= kCh; s1 -= kCh) {
            int f[kCh];
            double2 rd[kCh];
            double c[kCh], old[kCh], y[kCh];
#pragma unroll
            for (int k = 0; k < kCh; ++k) {
                const int s = s1 - k;
                f[k] = lt[s * LANES];
                rd[k] = col[s * LANES];
                c[k] = Cbw[s * LANES];
                old[k] = ty.crank ? Vw[s * LANES] : 0.0;
                y[k] = kri[s * LANES];
            }
#pragma unroll
            for (int k = 0; k < kCh; ++k) bwd(s1 - k, f[k], rd[k], c[k], old[k], true, y[k]);
        }
        for (; s1 >= 0; --s1)
            bwd(s1, lt[s1 * LANES], col[s1 * LANES], Cbw[s1 * LANES], ty.crank ? Vw[s1 * LANES] : 0.0, true,
                kri[s1 * LANES]);
        finite_check(v, xn, active);   // row 0's solution
        if (full && it == 0) {   // this tile's kept factors now match the fields
            __syncwarp();
            if (lane == 0) v.tgen[t] = sgen;
        }
        }
        }
    step_end:
        if (SPLIT) {
            if (bad) sbad = 1;
            bar_named(2, 2 * LANES);   // the step's Vm is written before the next step reads it
            if (sbad) return;
        } else if (bad) {
            return;
        }
    }
}

template <typename G>
cudaError_t stack_launch(const DevView &v, int tile0, int tile1, int cap, int nsteps, long long step, bool giv,
                         bool split, cudaStream_t st)
{
    split = split && !giv;
    const size_t smem = ((size_t)cap + (split ? 2 * kSplitRows : 0)) * LANES * sizeof(double);
    auto fn = giv ? k_stack<G, true, false> : split ? k_stack<G, false, true> : k_stack<G, false, false>;
    if (smem > 48 * 1024) {
        const cudaError_t ce = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (ce != cudaSuccess) return ce;
    }
    fn<<<tile1 - tile0, split ? 2 * LANES : LANES, smem, st>>>(v, tile0, tile1, cap, nsteps, step);
    return cudaGetLastError();
}

// ------------------------------------------------------------ wide tiles
// A wide tile holds one neuron; its compartments run on the threads of one
// block (slot s on thread s mod blockDim), its rows are contiguous (stride
// 1). Per step: the table cursors each compartment starts from are resolved
// first (the reference carries the bracket of the last NEWVOLT / NEWCONC1
// from one compartment to the next, hines_chip.c:174-203), then every
// compartment's program runs, the pool program runs on thread 0, and the
// elimination runs level by level: forward, a row pulls its children in
// ascending row order once they are final (the order the sequential sweep
// applies them in); backward, top-down from the root.
//
// Elimination schedule at DevView::wtop + Tile::wtop:
//   nf, fwd_start[nf+1], fwd_rows[S], kid_start[S+1], kids[S-1],
//   nb, bwd_start[nb+1], bwd_rows[S]

// Row of the table bracket a fresh lookup of v lands in (clamped).
__device__ __forceinline__ int fresh_row(double v, double vmin, double inv, int divs)
{
    double f = (v - vmin) * inv;
    if (f < 0.0) f = 0.0;
    else if (f > divs) f = divs;
    return (int)f;
}

__device__ __forceinline__ bool bracket_hit(const double *vals, int row, double v)
{
    return !((vals[row] > v) || (v >= vals[row + 1]));
}

__device__ __forceinline__ void cursor_at(VCursor &c, int row, const double *vals, int ncols)
{
    c.row = row;
    c.lo = vals[row];
    c.hi = vals[row + 1];
    c.base = row * ncols;
}

// Incoming bracket rows of one cursor chain: slots with prev[s] != -2 look
// the value val(s) up; prev[s] is the previous such slot (-1: none). Fresh
// lookups are exact unless a value sits in the previous bracket while its
// own fresh row differs (a rounding edge): then thread 0 replays the chain.
template <typename VAL>
__device__ __forceinline__ void cursor_chain(int S, const int *prev, VAL val, const double *vals, double vmin,
                                             double inv, int divs, int *fresh, int *in)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int s = tid; s < S; s += nt) fresh[s] = prev[s] != -2 ? fresh_row(val(s), vmin, inv, divs) : -1;
    __syncthreads();
    int edge = 0;
    for (int s = tid; s < S; s += nt) {
        if (prev[s] == -2) continue;
        const int r = prev[s] >= 0 ? fresh[prev[s]] : -1;
        if (r >= 0 && bracket_hit(vals, r, val(s)) && r != fresh[s]) edge = 1;
    }
    if (__syncthreads_or(edge)) {
        if (tid == 0) {
            int state = -1;
            for (int s = 0; s < S; ++s) {
                if (prev[s] == -2) continue;
                in[s] = state;
                const double x = val(s);
                if (state < 0 || !bracket_hit(vals, state, x)) state = fresh_row(x, vmin, inv, divs);
            }
        }
    } else {
        for (int s = tid; s < S; s += nt)
            if (prev[s] != -2) in[s] = prev[s] >= 0 ? fresh[prev[s]] : -1;
    }
    __syncthreads();
}

// Shared memory: 2*smax doubles (diagonal, right-hand side) + 4*smax ints.
// One warp per block (wide_threads); 128 registers a thread: the FP64
// interpreter spills at 80 (measured with 256-thread blocks: 513 against 841
// us/step on 10,000 random trees).
template <typename G, bool GIV>
__global__ void __launch_bounds__(32, 16)
k_wide(DevView v, int tile0, int tile1, int smax, int nsteps, long long step0)
{
    extern __shared__ double sm[];
    const int t = tile0 + blockIdx.x;
    if (t >= tile1) return;
    const int tid = threadIdx.x, nt = blockDim.x;
    const long long sbase = v.step_dev ? *v.step_dev : 0;
    const Tile tl = v.tiles[t];
    const TileType ty = v.types[tl.type];
    const TableGeom tg = v.tgeom[ty.table_set];
    const int S = ty.nslots;
    double *Ds = sm, *Rs = sm + smax;
    int *vfresh = reinterpret_cast<int *>(sm + 2 * smax), *vin = vfresh + smax, *cfresh = vin + smax,
        *cin = cfresh + smax;
    const int *meta = v.prog + ty.wide_off;
    const int *sofs = meta, *vprev = meta + S, *cprev = meta + 2 * S, *cpool = meta + 3 * S;
    const int *wt = v.wtop + tl.wtop;
    const int nf = wt[0];
    const int *fst = wt + 1, *frows = fst + nf + 1, *kst = frows + S, *kids = kst + S + 1;
    const int nb = kids[S - 1];
    const int *bst = kids + S, *brows = bst + nb + 1;

    double *P = v.P + tl.fld * LANES;
    double *V = v.V + tl.vm * LANES;
    double *C = v.C + tl.pools * LANES;
    const int *par = v.parent + tl.topo * LANES;
    const double *A = v.A + tl.topo * LANES, *B = v.B + tl.topo * LANES, *Cb = v.Cb + tl.topo * LANES;

    ChanEnv<G> E;
    E.tab = tab_ptr<G>(v, tg.tab_off);
    E.xvals = v.xyvals + tg.xv_off;
    E.yvals = tg.yv_off >= 0 ? v.xyvals + tg.yv_off : E.xvals;
    E.tg = tg;
    E.ncols = tg.ncols;
    E.interp = ty.interp != 0;
    E.c5 = ty.chanmode5 != 0;
    E.has_cd = ty.has_cd != 0;
    ChanRows NR;
    NR.P = P;
    NR.I = v.I + tl.ints * LANES;
    NR.C = C;
    NR.F = v.F + tl.pools * LANES;
    NR.G = v.giv + tl.giv * LANES;
    NR.CD = v.CD ? v.CD + tl.pools * LANES : nullptr;
    NR.IT = nullptr;   // storemode types never run wide
    NR.ring = v.ring + tl.syn * LANES;
    NR.neuron = tl.first_neuron;
    NR.active = true;

    for (int it = 0; it < nsteps; ++it) {
        const long long step = sbase + step0 + it;
        if (tg.ncols) {
            cursor_chain(S, vprev, [&](int s) { return V[s]; }, E.xvals, tg.xmin, tg.invdx, tg.xdivs, vfresh, vin);
            cursor_chain(S, cprev, [&](int s) { return C[cpool[s]]; }, E.yvals, tg.ymin, tg.invdy, tg.ydivs, cfresh,
                         cin);
        }
        // channel phase
        for (int s = tid; s < S; s += nt) {
            ChanState cs;
            chan_state_reset(cs, tg.ncols);
            if (tg.ncols && vprev[s] != -2 && vin[s] >= 0) cursor_at(cs.vc, vin[s], E.xvals, tg.ncols);
            if (tg.ncols && cprev[s] != -2 && cin[s] >= 0) {
                cursor_at(cs.cc, cin[s], E.yvals, tg.ncols);
                cs.ctab_base = cs.cc.base;
            }
            const int *pc = v.prog + sofs[s];
            double R = 0.0, D = 1.0;
            if (!chan_compartment<G, GIV, 1>(v, E, cs, NR, pc, V[s], step, R, D) && v.status)
                atomicOr(v.status, ST_BAD_OP);
            Rs[s] = R;
            Ds[s] = D;
        }
        __syncthreads();
        if (tid == 0) {
            PoolLane PL;
            PL.C = C;
            PL.F = NR.F;
            PL.CR = v.CR ? v.CR + tl.pools * LANES : nullptr;
            PL.CD = NR.CD;
            PL.S = v.S ? v.S + tl.scr * LANES : nullptr;
            PL.P = P;
            PL.V = V;
            PL.dt = v.dt;
            PL.crank = ty.crank;
            if (!pool_phase<1>(v.prog + ty.pool_off, PL) && v.status) atomicOr(v.status, ST_BAD_OP);
        }
        __syncthreads();
        // forward elimination, leaves first
        for (int l = 0; l < nf; ++l) {
            for (int i = fst[l] + tid; i < fst[l + 1]; i += nt) {
                const int s = frows[i];
                double d = Ds[s], r = Rs[s];
                for (int k = kst[s]; k < kst[s + 1]; ++k) {
                    const int c = kids[k];
                    const double temp = A[c] / Ds[c];
                    d -= B[c] * temp;
                    r -= Rs[c] * temp;
                }
                Ds[s] = d;
                Rs[s] = r;
            }
            __syncthreads();
        }
        // back substitution, root first
        for (int l = 0; l < nb; ++l) {
            for (int i = bst[l] + tid; i < bst[l + 1]; i += nt) {
                const int s = brows[i];
                const int p = par[s];
                double r = Rs[s];
                if (p >= 0) r -= Cb[s] * Rs[p];
                r = r / Ds[s];
                Rs[s] = r;
                if (ty.crank) {
                    const double old = V[s];
                    V[s] = r + r - old;
                } else {
                    V[s] = r;
                }
            }
            __syncthreads();
        }
        if (tid == 0) finite_check(v, V[0], true);
    }
}

cudaError_t launch_fp64_wide(const DevView &v, int tile0, int tile1, int smax, int nsteps, long long step, bool giv,
                             cudaStream_t st);
cudaError_t launch_mixed_wide(const DevView &v, int tile0, int tile1, int smax, int nsteps, long long step, bool giv,
                              cudaStream_t st);

inline size_t wide_smem(int smax) { return (size_t)smax * (2 * sizeof(double) + 4 * sizeof(int)); }
// One warp per neuron: a warp's __syncthreads is cheap, and many small
// blocks hide each other's waits (10,000 random trees, mixed: 146 us/step
// with 32 threads, 154 with 64, 199 with 128, 216 with 256; FP64 332 / 348 /
// 409 / 539).
inline int wide_threads(int) { return 32; }

template <typename KF>
cudaError_t wide_launch(KF fn, const DevView &v, int tile0, int tile1, int smax, int nsteps, long long step,
                        cudaStream_t st)
{
    const size_t smem = wide_smem(smax);
    if (smem > 48 * 1024) {
        const cudaError_t ce = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (ce != cudaSuccess) return ce;
    }
    fn<<<tile1 - tile0, wide_threads(smax), smem, st>>>(v, tile0, tile1, smax, nsteps, step);
    return cudaGetLastError();
}

// Launchers, one per precision translation unit (the FP64 unit is compiled
// without multiply-add contraction, the mixed unit with it).
cudaError_t launch_fp64(const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                        long long step, bool giv, cudaStream_t st);
cudaError_t launch_mixed(const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                         long long step, bool giv, cudaStream_t st);

// Stack elimination tiles (TileType::stack), one warp per tile (mixed form,
// split: two, see k_stack_mixed), cap doubles of shared memory per lane.
cudaError_t launch_fp64_stack(const DevView &v, int tile0, int tile1, int cap, int nsteps, long long step, bool giv,
                              bool split, cudaStream_t st);
cudaError_t launch_mixed_stack(const DevView &v, int tile0, int tile1, int cap, int nsteps, long long step,
                               bool giv, bool split, cudaStream_t st);

// Cooperative multi-step launch over tiles [0, ntiles), one warp per block,
// with a grid barrier after every step (v.gbar set): every block must be
// resident at once, otherwise cudaErrorCooperativeLaunchTooLarge.
cudaError_t launch_fp64_coop(const DevView &v, int ntiles, int smax, int nsteps, long long step, cudaStream_t st);
cudaError_t launch_mixed_coop(const DevView &v, int ntiles, int smax, int nsteps, long long step, cudaStream_t st);

template <typename Fn>
cudaError_t coop_launch(Fn fn, const DevView &v, int ntiles, int smax, int nsteps, long long step, cudaStream_t st)
{
    const size_t smem = (size_t)2 * smax * LANES * sizeof(double);
    cudaError_t ce;
    if (smem > 48 * 1024) {
        ce = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (ce != cudaSuccess) return ce;
    }
    int dev = 0, nsm = 0, per_sm = 0;
    if ((ce = cudaGetDevice(&dev)) != cudaSuccess) return ce;
    if ((ce = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return ce;
    if ((ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, LANES, smem)) != cudaSuccess) return ce;
    if ((long long)per_sm * nsm < ntiles) return cudaErrorCooperativeLaunchTooLarge;
    DevView vv = v;
    int t0 = 0, t1 = ntiles;
    void *args[] = {&vv, &t0, &t1, &smax, &nsteps, &step};
    return cudaLaunchCooperativeKernel((const void *)fn, dim3(ntiles), dim3(LANES), args, smem, st);
}

template <typename G>
cudaError_t launch_impl(const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                        long long step, bool giv, cudaStream_t st)
{
    const int ntiles = tile1 - tile0;
    const int blocks = (ntiles + warps - 1) / warps;
    const size_t smem = (size_t)warps * 2 * smax * LANES * sizeof(double);
    cudaError_t ce;
    if (giv) {
        if (smem > 48 * 1024) {
            ce = cudaFuncSetAttribute(k_steps<G, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (ce != cudaSuccess) return ce;
        }
        k_steps<G, true><<<blocks, warps * LANES, smem, st>>>(v, tile0, tile1, smax, nsteps, step);
    } else {
        if (smem > 48 * 1024) {
            ce = cudaFuncSetAttribute(k_steps<G, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (ce != cudaSuccess) return ce;
        }
        k_steps<G, false><<<blocks, warps * LANES, smem, st>>>(v, tile0, tile1, smax, nsteps, step);
    }
    return cudaGetLastError();
}

}  // namespace gbh
