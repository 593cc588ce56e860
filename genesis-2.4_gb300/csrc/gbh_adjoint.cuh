// gbh_adjoint.cuh -- reverse-mode (adjoint) kernels of the FP64 form.
//
// Loss L = sum over steps n and target rows j of (Vm_j after step n - trace[n][j])^2.
// The reference has no gradient; this is the differentiated form of its step
// (do_chip_hh4_update, genesis/src/hines/hines_chip.c:157-600, followed by
// do_euler_hsolve / do_crank_hsolve, genesis/src/hines/hines_solve.c:140-296).
//
// Checkpointed reverse sweep. k_adj_forward runs the forward step on work
// copies of the state; in checkpoint mode it stores Vm and the gate states
// every K steps, in tape mode it restarts from one checkpoint and records, for
// each of the next K steps, the values the reverse step needs: Vm before the
// step, each row's diagonal D' and rhs R' after forward elimination, the
// solution x, and the gate states before the step. k_adj_reverse then walks
// those steps backwards:
//   1. seed: the adjoint of Vm after the step gains 2*(Vm - target) at target
//      rows (Crank-Nicolson: Vm_after = 2x - Vm_before);
//   2. back substitution reversed, rows ascending (a row's adjoint is final
//      once its children, the lower rows, have pushed into it):
//      x_s = (R'_s - C_s x_p) / D'_s;
//   3. forward elimination reversed, rows descending:
//      t_s = A_s / D'_s, D'_p -= B_s t_s, R'_p -= R'_s t_s;
//   4. channel program reversed per compartment: rhs = Vm + ichan*tbyc,
//      diag = sumg*tbyc + diagterm, ichan = Em/Rm + inject + sum Ek*G,
//      G = gmax * prod x^p, the trapezoid gate update x' = (x(2-B') + A')/B'
//      (x' = A'/B' for instantaneous gates) and the linear table
//      interpolation, whose derivative in Vm is the interval slope times
//      1/dx (zero where the lookup clamps at either end of the table, and
//      zero without interpolation).
// Outputs: adjoints of Vm and of the gate states before the first step, and
// accumulated gradients of every parameter field (Em/Rm, inject, Ek, gmax,
// tbyc, diagterm) and of the three elimination coefficients of every row.
// Supported programs: compartments with voltage-table gated channels
// (M_BEGIN, M_NEWVOLT, M_CHAN, M_CHAN_G, M_GATE of kind GK_1V with a nonzero
// power, M_ADDCURR, M_END); the host rejects anything else.
#pragma once
#include <cuda_runtime.h>
#include "gbh_devfn.cuh"
#include "gbh_adjoint.h"

namespace gbh {

struct AdjLane {
    const int *prog;
    int S;
    bool interp, crank;
    const double *tab, *xvals;
    TableGeom tg;
    double *P, *V;
    const int *par;
    const double *A, *B, *C;
};

__device__ __forceinline__ AdjLane adj_lane(const AdjView &v, const Tile &tl, int lane)
{
    const TileType ty = v.types[tl.type];
    AdjLane a;
    a.prog = v.prog + ty.prog_off;
    a.S = ty.nslots;
    a.interp = ty.interp != 0;
    a.crank = ty.crank != 0;
    a.tg = v.tgeom[ty.table_set];
    a.tab = v.tab64 + a.tg.tab_off;
    a.xvals = v.xyvals + a.tg.xv_off;
    a.P = v.P + tl.fld * LANES + lane;
    a.V = v.V + tl.vm * LANES + lane;
    a.par = v.parent + tl.topo * LANES + lane;
    a.A = v.A + tl.topo * LANES + lane;
    a.B = v.B + tl.topo * LANES + lane;
    a.C = v.Cb + tl.topo * LANES + lane;
    return a;
}

__device__ __forceinline__ void adj_cursor_reset(VCursor &vc, int ncols)
{
    if (ncols) { vc.lo = vc.hi = 0.0; } else { vc.lo = -1e20; vc.hi = 1e20; }
    vc.row = vc.base = 0;
    vc.frac = 0.0;
}

// Operand count + 1 of the micro-ops the differentiated form accepts.
__device__ __forceinline__ int adj_op_len(int code)
{
    switch (code) {
    case M_BEGIN: case M_GATE: return 5;
    case M_END: return 4;
    case M_CHAN: return 3;
    case M_NEWVOLT: return 1;
    default: return 2;   // M_CHAN_G, M_ADDCURR
    }
}

// locate() of the interpolating lookup, also reporting whether the fraction
// moves with v (false where a fresh lookup clamps at either end of the table).
__device__ __forceinline__ bool locate_lin(VCursor &c, double v, const TableGeom &tg, const double *vals)
{
    double f = (v - tg.xmin) * tg.invdx;
    bool lin = true;
    if ((c.lo > v) || (v >= c.hi)) {
        if (f < 0.0) {
            f = 0.0;
            lin = false;
        } else if (f > tg.xdivs) {
            f = tg.xdivs;
            lin = false;
        }
        c.row = (int)f;
        f = f - (double)c.row;
        c.lo = vals[c.row];
        c.hi = vals[c.row + 1];
        c.base = c.row * tg.ncols;
    } else {
        f = f - (double)c.row;
    }
    c.frac = f;
    return lin;
}

// One forward step of the lane's neuron on the work arrays; arithmetic and
// operand order as the engine's FP64 step. With tp != nullptr it records the
// step's tape rows (Vm, D', R', x, gate states before the update).
__device__ __forceinline__ bool adj_forward_step(const AdjLane &a, double *Dc, double *Rc, double *tp)
{
    const int S = a.S;
    const int ncols = a.tg.ncols;
    VCursor vc;
    adj_cursor_reset(vc, ncols);
    double Ek = 0.0, Gk = 0.0;
    int gi = 0;
    const int *pc = a.prog;
    for (int s = 0; s < S; ++s) {
        const double Vm = a.V[s * LANES];
        if (tp) tp[s * LANES] = Vm;
        double sumg = 0.0, ichan = 0.0;
        for (;;) {
            const int code = pc[0];
            if (code == M_BEGIN) {
                ichan = a.P[pc[1] * LANES] + a.P[pc[2] * LANES];
                pc += 5;
            } else if (code == M_NEWVOLT) {
                locate(vc, Vm, a.tg.xmin, a.tg.invdx, a.tg.xdivs, a.xvals, ncols, a.interp);
                pc += 1;
            } else if (code == M_CHAN) {
                Ek = a.P[pc[1] * LANES];
                Gk = a.P[pc[2] * LANES];
                pc += 3;
            } else if (code == M_CHAN_G) {
                Gk = a.P[pc[1] * LANES];
                pc += 2;
            } else if (code == M_GATE) {
                const int b = vc.base + pc[2];
                double X, Y;
                if (a.interp) {
                    const double fr = vc.frac;
                    X = a.tab[b];
                    X = X + fr * (a.tab[b + ncols] - X);
                    Y = a.tab[b + 1];
                    Y = Y + fr * (a.tab[b + 1 + ncols] - Y);
                } else {
                    X = a.tab[b];
                    Y = a.tab[b + 1];
                }
                const int p = pc[3];
                double *st = &a.P[pc[4] * LANES];
                if (tp) tp[(4 * S + gi) * LANES] = *st;
                ++gi;
                double x;
                int pw = p;
                if (p > 0) {
                    x = (*st * (2.0 - X) + Y) / X;
                } else {
                    x = Y / X;
                    pw = -p;
                }
                *st = x;
                Gk = gpow<double>(Gk, x, pw);
                pc += 5;
            } else if (code == M_ADDCURR) {
                sumg += Gk;
                ichan += Ek * Gk;
                pc += 2;
            } else if (code == M_END) {
                const double tbyc = a.P[pc[1] * LANES];
                Rc[s * LANES] = Vm + ichan * tbyc;
                Dc[s * LANES] = sumg * tbyc + a.P[pc[2] * LANES];
                pc += 4;
                break;
            } else {
                return false;
            }
        }
    }
    for (int s = 0; s < S; ++s) {
        const int p = a.par[s * LANES];
        if (tp) {
            tp[(S + s) * LANES] = Dc[s * LANES];
            tp[(2 * S + s) * LANES] = Rc[s * LANES];
        }
        if (p >= 0) {
            const double temp = a.A[s * LANES] / Dc[s * LANES];
            Dc[p * LANES] -= a.B[s * LANES] * temp;
            Rc[p * LANES] -= Rc[s * LANES] * temp;
        }
    }
    for (int s = S - 1; s >= 0; --s) {
        const int p = a.par[s * LANES];
        double r = Rc[s * LANES];
        if (p >= 0) r -= a.C[s * LANES] * Rc[p * LANES];
        r = r / Dc[s * LANES];
        Rc[s * LANES] = r;
        if (tp) tp[(3 * S + s) * LANES] = r;
        if (a.crank) {
            const double old = a.V[s * LANES];
            a.V[s * LANES] = r + r - old;
        } else {
            a.V[s * LANES] = r;
        }
    }
    return true;
}

// Copies Vm and the gate states between the work arrays and a checkpoint block.
__device__ __forceinline__ void adj_checkpoint(const AdjLane &a, double *ck, bool save)
{
    const int S = a.S;
    for (int s = 0; s < S; ++s) {
        if (save) ck[s * LANES] = a.V[s * LANES];
        else a.V[s * LANES] = ck[s * LANES];
    }
    int gi = 0;
    const int *pc = a.prog;
    for (int s = 0; s < S; ++s) {
        for (;;) {
            const int code = pc[0];
            if (code == M_GATE) {
                double *st = &a.P[pc[4] * LANES];
                if (save) ck[(S + gi) * LANES] = *st;
                else *st = ck[(S + gi) * LANES];
                ++gi;
            }
            pc += adj_op_len(code);
            if (code == M_END) break;
        }
    }
}

// mode 0: run nsteps steps from the work state, saving checkpoint c before
//         every step with step % K == 0 and after the last one when nsteps
//         is a multiple of K (c = step / K);
// mode 1: restore checkpoint seg, then run nsteps (<= K) steps recording the tape.
__global__ void __launch_bounds__(32)
k_adj_forward(AdjView v, int tile0, int tile1, int smax, int nsteps, int K, int mode, int seg)
{
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31;
    const int t = tile0 + blockIdx.x;
    if (t >= tile1) return;
    const Tile tl = v.tiles[t];
    const AdjLane a = adj_lane(v, tl, lane);
    double *Dc = sm + lane;
    double *Rc = Dc + (size_t)smax * LANES;
    if (mode == 1) adj_checkpoint(a, v.ckpt + ((int64_t)seg * v.ck_stride + v.ck_off[t]) * LANES + lane, false);
    for (int k = 0; k < nsteps; ++k) {
        double *tp = nullptr;
        if (mode == 0) {
            if (k % K == 0)
                adj_checkpoint(a, v.ckpt + ((int64_t)(k / K) * v.ck_stride + v.ck_off[t]) * LANES + lane, true);
        } else {
            tp = v.tape + ((int64_t)k * v.tp_stride + v.tp_off[t]) * LANES + lane;
        }
        if (!adj_forward_step(a, Dc, Rc, tp)) {
            if (v.status) atomicOr(v.status, ST_BAD_OP);
            return;
        }
    }
    if (mode == 0 && nsteps % K == 0)
        adj_checkpoint(a, v.ckpt + ((int64_t)(nsteps / K) * v.ck_stride + v.ck_off[t]) * LANES + lane, true);
}

// Reverse of tape steps nk-1 .. 0 of one segment; step0 = global index of its
// first step (row of the trace).
__global__ void __launch_bounds__(32)
k_adj_reverse(AdjView v, int tile0, int tile1, int smax, int nk, int step0)
{
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31;
    const int t = tile0 + blockIdx.x;
    if (t >= tile1) return;
    const Tile tl = v.tiles[t];
    const AdjLane a = adj_lane(v, tl, lane);
    const int S = a.S;
    const int ncols = a.tg.ncols;
    double *Vb = v.Vbar + tl.vm * LANES + lane;
    double *Xb = v.Xbar + tl.fld * LANES + lane;
    double *Gf = v.Gf + tl.fld * LANES + lane;
    double *GA = v.GA + tl.topo * LANES + lane;
    double *GB = v.GB + tl.topo * LANES + lane;
    double *GC = v.GC + tl.topo * LANES + lane;
    const int *tgt = v.tgt + tl.topo * LANES + lane;
    double *Db = sm + lane;                    // adjoint of D' (final), then of the initial diag
    double *Rb = Db + (size_t)smax * LANES;    // adjoint of x, then of R
    double *loss = v.loss + (size_t)t * LANES + lane;

    for (int k = nk - 1; k >= 0; --k) {
        const double *tp = v.tape + ((int64_t)k * v.tp_stride + v.tp_off[t]) * LANES + lane;
        const double *tV = tp, *tD = tp + (size_t)S * LANES, *tR = tp + (size_t)2 * S * LANES,
                     *tX = tp + (size_t)3 * S * LANES, *tG = tp + (size_t)4 * S * LANES;
        const double *trow = v.trace + (size_t)(step0 + k) * v.ntargets;
        // ---- 1. seed (the loss is summed step by step, descending, so the
        //      total does not depend on the checkpoint interval) ----
        double lstep = 0.0;
        for (int s = 0; s < S; ++s) {
            double vb = Vb[s * LANES];
            const int j = tgt[s * LANES];
            if (j >= 0) {
                const double x = tX[s * LANES];
                const double vnext = a.crank ? x + x - tV[s * LANES] : x;
                const double diff = vnext - trow[j];
                lstep += diff * diff;
                vb += 2.0 * diff;
            }
            Rb[s * LANES] = a.crank ? 2.0 * vb : vb;
            Vb[s * LANES] = a.crank ? -vb : 0.0;
        }
        *loss += lstep;
        // ---- 2. back substitution reversed ----
        for (int s = 0; s < S; ++s) {
            const int p = a.par[s * LANES];
            const double rb = Rb[s * LANES] / tD[s * LANES];
            Rb[s * LANES] = rb;
            if (p >= 0) {
                Rb[p * LANES] -= a.C[s * LANES] * rb;
                GC[s * LANES] -= tX[p * LANES] * rb;
            }
            Db[s * LANES] = -tX[s * LANES] * rb;
        }
        // ---- 3. forward elimination reversed ----
        for (int s = S - 1; s >= 0; --s) {
            const int p = a.par[s * LANES];
            if (p < 0) continue;
            const double d = tD[s * LANES];
            const double tt = a.A[s * LANES] / d;
            const double dbp = Db[p * LANES], rbp = Rb[p * LANES];
            const double tb = -a.B[s * LANES] * dbp - tR[s * LANES] * rbp;
            GB[s * LANES] -= tt * dbp;
            Rb[s * LANES] -= tt * rbp;
            const double tbd = tb / d;
            GA[s * LANES] += tbd;
            Db[s * LANES] -= tt * tbd;
        }
        // ---- 4. channel program reversed ----
        VCursor vc;
        adj_cursor_reset(vc, ncols);
        double Ek = 0.0, gmax = 0.0, dfdv = 0.0;
        int fEk = -1, fG = -1, ng = 0, gi = 0;
        int gf[ADJ_MAX_GATES], gp[ADJ_MAX_GATES];
        double gX[ADJ_MAX_GATES], gsX[ADJ_MAX_GATES], gsY[ADJ_MAX_GATES], gst[ADJ_MAX_GATES],
            gx[ADJ_MAX_GATES];
        const int *pc = a.prog;
        for (int s = 0; s < S; ++s) {
            const double Vm = tV[s * LANES];
            const double rb = Rb[s * LANES], db = Db[s * LANES];
            const int *q = pc;
            while (q[0] != M_END) q += adj_op_len(q[0]);
            const double tbyc = a.P[q[1] * LANES];
            const double Ibar = rb * tbyc, Sbar = db * tbyc;
            double vbn = Vb[s * LANES] + rb;
            double sumg = 0.0, ichan = 0.0;
            for (;;) {
                const int code = pc[0];
                if (code == M_BEGIN) {
                    Gf[pc[1] * LANES] += Ibar;
                    Gf[pc[2] * LANES] += Ibar;
                    ichan = a.P[pc[1] * LANES] + a.P[pc[2] * LANES];
                    pc += 5;
                } else if (code == M_NEWVOLT) {
                    if (a.interp) {
                        dfdv = locate_lin(vc, Vm, a.tg, a.xvals) ? a.tg.invdx : 0.0;
                    } else {
                        locate(vc, Vm, a.tg.xmin, a.tg.invdx, a.tg.xdivs, a.xvals, ncols, false);
                        dfdv = 0.0;
                    }
                    pc += 1;
                } else if (code == M_CHAN || code == M_CHAN_G) {
                    if (code == M_CHAN) {
                        fEk = pc[1];
                        Ek = a.P[pc[1] * LANES];
                        fG = pc[2];
                        pc += 3;
                    } else {
                        fG = pc[1];
                        pc += 2;
                    }
                    gmax = a.P[fG * LANES];
                    ng = 0;
                } else if (code == M_GATE) {
                    const int b = vc.base + pc[2];
                    double X, Y, sX = 0.0, sY = 0.0;
                    if (a.interp) {
                        const double fr = vc.frac;
                        X = a.tab[b];
                        sX = a.tab[b + ncols] - X;
                        X = X + fr * sX;
                        Y = a.tab[b + 1];
                        sY = a.tab[b + 1 + ncols] - Y;
                        Y = Y + fr * sY;
                    } else {
                        X = a.tab[b];
                        Y = a.tab[b + 1];
                    }
                    const int p = pc[3];
                    const double st = tG[gi * LANES];
                    ++gi;
                    if (ng < ADJ_MAX_GATES) {
                        gf[ng] = pc[4];
                        gp[ng] = p;
                        gX[ng] = X;
                        gsX[ng] = sX * dfdv;
                        gsY[ng] = sY * dfdv;
                        gst[ng] = st;
                        gx[ng] = p > 0 ? (st * (2.0 - X) + Y) / X : Y / X;
                        ++ng;
                    } else if (v.status) {
                        atomicOr(v.status, ST_BAD_OP);
                    }
                    pc += 5;
                } else if (code == M_ADDCURR) {
                    double prod = 1.0;
                    for (int g = 0; g < ng; ++g) prod = gpow<double>(prod, gx[g], gp[g] > 0 ? gp[g] : -gp[g]);
                    const double G = gmax * prod;
                    sumg += G;
                    ichan += Ek * G;
                    const double Gbar = Sbar + Ibar * Ek;
                    if (fEk >= 0) Gf[fEk * LANES] += Ibar * G;
                    Gf[fG * LANES] += Gbar * prod;
                    for (int g = 0; g < ng; ++g) {
                        const int pw = gp[g] > 0 ? gp[g] : -gp[g];
                        double others = 1.0;
                        for (int h = 0; h < ng; ++h)
                            if (h != g) others = gpow<double>(others, gx[h], gp[h] > 0 ? gp[h] : -gp[h]);
                        double xpm1 = 1.0;
                        for (int e = 1; e < pw; ++e) xpm1 *= gx[g];
                        const double xhat = Xb[gf[g] * LANES] + Gbar * gmax * (double)pw * xpm1 * others;
                        const double rX = 1.0 / gX[g];
                        const double Abar = xhat * rX;
                        double Bbar, xbn;
                        if (gp[g] > 0) {
                            Bbar = -xhat * (gx[g] + gst[g]) * rX;
                            xbn = xhat * (2.0 - gX[g]) * rX;
                        } else {
                            Bbar = -xhat * gx[g] * rX;
                            xbn = 0.0;
                        }
                        vbn += Abar * gsY[g] + Bbar * gsX[g];
                        Xb[gf[g] * LANES] = xbn;
                    }
                    ng = 0;
                    pc += 2;
                } else if (code == M_END) {
                    Gf[pc[1] * LANES] += rb * ichan + db * sumg;
                    Gf[pc[2] * LANES] += db;
                    pc += 4;
                    break;
                } else {
                    if (v.status) atomicOr(v.status, ST_BAD_OP);
                    return;
                }
            }
            Vb[s * LANES] = vbn;
        }
    }
}

}  // namespace gbh
