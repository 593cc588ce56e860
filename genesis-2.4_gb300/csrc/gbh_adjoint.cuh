// gbh_adjoint.cuh -- reverse-mode (adjoint) kernels of the FP64 form.
//
// Loss L = sum over steps n and target rows j of (Vm_j after step n - trace[n][j])^2.
// The reference has no gradient; this is the differentiated form of its step
// (do_chip_hh4_update, genesis/src/hines/hines_chip.c:157-600, followed by
// do_euler_hsolve / do_crank_hsolve, genesis/src/hines/hines_solve.c:140-296).
//
// FP64 arithmetic on GB300: one warp issues at most ~0.47 lane-DFMA per clock
// whether its lanes are active or not, an SM ~1.6 with four warps or more, so
// a batch of a few thousand neurons (one warp per 32) reaches a quarter of the
// GPU's FP64 rate in any kernel that walks the steps one after another. The
// sweep therefore keeps the sequential kernels lean and moves the rest into
// kernels that are parallel over steps as well as neurons:
//
//   forward   the engine's own step kernel advances work copies of Vm and the
//             gate states; k_adj_copy stores them every K steps (checkpoints)
//             and, when a segment is recomputed, before every step (snapshot);
//   k_adj_linearize   (parallel over steps) recomputes each step of a segment
//             from its snapshot with the step's exact arithmetic and stores
//             the local derivatives the reverse needs: 1/D', A/D', R' and x of
//             every row, ichan and sumg of every compartment, the gate product
//             of every channel, and per gate d prod/dx, dx'/dVm (table slope,
//             zero where the lookup clamps or without interpolation) and
//             dx'/dx (the trapezoid factor (2-B')/B', zero for instant gates);
//   k_adj_reverse   (sequential over steps, one lane per neuron; the tree
//             walk on one warp, the channel phase spread over four) the
//             adjoint recurrence of Vm and the gate states:
//               seed      Vm-bar += 2 (Vm after - target) at target rows
//                         (Crank-Nicolson: Vm after = 2x - Vm before);
//               back substitution reversed, rows ascending:
//                         x_s = (R'_s - C_s x_p) / D'_s;
//               forward elimination reversed, rows descending:
//                         t_s = A_s / D'_s, D'_p -= B_s t_s, R'_p -= R'_s t_s;
//               channels  rhs = Vm + ichan*tbyc, diag = sumg*tbyc + diagterm,
//                         G = gmax prod x^p, x' = (x(2-B') + A')/B';
//             it stores the adjoints of R, D and of the back substitution;
//   k_adj_reduce   (parallel over rows) sums the parameter gradients of a
//             segment from those adjoints and the tape, steps descending so
//             the totals do not depend on the checkpoint interval.
// Supported programs: compartments with voltage-table gated channels
// (M_BEGIN, M_NEWVOLT, M_CHAN, M_CHAN_G, M_GATE of kind GK_1V with a nonzero
// power, M_ADDCURR, M_END); the host rejects anything else.
#pragma once
#include <cuda_runtime.h>
#include "gbh_devfn.cuh"
#include "gbh_adjoint.h"

namespace gbh {

__device__ __forceinline__ double *adj_tape(const AdjView &v, int k, int t, int lane)
{
    return v.tape + ((int64_t)k * v.tp_stride + v.tp_off[t]) * LANES + lane;
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

// ---------------------------------------------------------------- copies
// grid (tiles, row chunks of 32), 32 threads: one lane each.
__global__ void __launch_bounds__(32)
k_adj_copy(AdjView v, int c, int dir, int to_tape)
{
    const int lane = threadIdx.x;
    const int t = blockIdx.x;
    const Tile tl = v.tiles[t];
    const AdjType at = v.atypes[tl.type];
    const int rows = at.nslots + at.ngates;
    const int r0 = blockIdx.y * 32;
    const int r1 = min(rows, r0 + 32);
    double *blk = to_tape ? adj_tape(v, c, t, lane)
                          : v.ckpt + ((int64_t)c * v.ck_stride + v.ck_off[t]) * LANES + lane;
    for (int r = r0; r < r1; ++r) {
        double *w = r < at.nslots ? v.V + (tl.vm + r) * LANES + lane
                                  : v.P + (tl.fld + v.snap_field[at.snap_off + r - at.nslots]) * LANES + lane;
        if (dir == 0) blk[r * LANES] = *w;
        else *w = blk[r * LANES];
    }
}

// Checkpoint c0 + k -> tape step k (blockIdx.z = k): the snapshot rows of a
// segment whose every step was kept by the forward pass.
__global__ void __launch_bounds__(LANES)
k_adj_ck_to_tape(AdjView v, int c0)
{
    const int lane = threadIdx.x;
    const int t = blockIdx.x;
    const int k = blockIdx.z;
    const Tile tl = v.tiles[t];
    const AdjType at = v.atypes[tl.type];
    const int rows = at.nslots + at.ngates;
    const int r0 = blockIdx.y * 32;
    const int r1 = min(rows, r0 + 32);
    const double *src = v.ckpt + ((int64_t)(c0 + k) * v.ck_stride + v.ck_off[t]) * LANES + lane;
    double *dst = adj_tape(v, k, t, lane);
    for (int r = r0; r < r1; ++r) dst[r * LANES] = src[r * LANES];
}

// ---------------------------------------------------------------- linearisation
// grid (tiles, steps), 32 threads. Shared memory: 2 * smax * 32 doubles.
__global__ void __launch_bounds__(32)
k_adj_linearize(AdjView v, int smax)
{
    extern __shared__ double sm[];
    const int lane = threadIdx.x;
    const int t = blockIdx.x;
    const int k = blockIdx.y;
    const Tile tl = v.tiles[t];
    const TileType ty = v.types[tl.type];
    const AdjType at = v.atypes[tl.type];
    const TableGeom tg = v.tgeom[ty.table_set];
    const double *tab = v.tab64 + tg.tab_off;
    const double *xvals = v.xyvals + tg.xv_off;
    const int ncols = tg.ncols;
    const bool interp = ty.interp != 0;
    const int S = at.nslots;
    const AdjRows R = adj_rows(S, at.ngates, at.nchans);
    const double *P = v.P + tl.fld * LANES + lane;
    const int *par = v.parent + tl.topo * LANES + lane;
    const double *Aw = v.A + tl.topo * LANES + lane;
    const double *Bw = v.B + tl.topo * LANES + lane;
    const double *Cw = v.Cb + tl.topo * LANES + lane;
    double *tp = adj_tape(v, k, t, lane);
    double *Dc = sm + lane;
    double *Rc = Dc + (size_t)smax * LANES;

    VCursor vc;
    if (ncols) { vc.lo = vc.hi = 0.0; } else { vc.lo = -1e20; vc.hi = 1e20; }
    vc.row = vc.base = 0;
    vc.frac = 0.0;
    double dfdv = 0.0;
    double Ek = 0.0, Gk = 0.0;
    int gi = 0, ci = -1, cg0 = 0;
    double gx[ADJ_MAX_GATES];
    int gp[ADJ_MAX_GATES];
    const int *pc = v.prog + ty.prog_off;
    for (int s = 0; s < S; ++s) {
        const double Vm = tp[(R.V + s) * LANES];
        double sumg = 0.0, ichan = 0.0;
        for (;;) {
            const int code = pc[0];
            if (code == M_BEGIN) {
                ichan = P[pc[1] * LANES] + P[pc[2] * LANES];
                pc += 5;
            } else if (code == M_NEWVOLT) {
                if (interp) {
                    dfdv = locate_lin(vc, Vm, tg, xvals) ? tg.invdx : 0.0;
                } else {
                    locate(vc, Vm, tg.xmin, tg.invdx, tg.xdivs, xvals, ncols, false);
                    dfdv = 0.0;
                }
                pc += 1;
            } else if (code == M_CHAN || code == M_CHAN_G) {
                if (code == M_CHAN) {
                    Ek = P[pc[1] * LANES];
                    Gk = P[pc[2] * LANES];
                    pc += 3;
                } else {
                    Gk = P[pc[1] * LANES];
                    pc += 2;
                }
                ++ci;
                cg0 = gi;
            } else if (code == M_GATE) {
                const int b = vc.base + pc[2];
                double X, Y, sX = 0.0, sY = 0.0;
                if (interp) {
                    const double fr = vc.frac;
                    X = tab[b];
                    sX = tab[b + ncols] - X;
                    X = X + fr * sX;
                    Y = tab[b + 1];
                    sY = tab[b + 1 + ncols] - Y;
                    Y = Y + fr * sY;
                } else {
                    X = tab[b];
                    Y = tab[b + 1];
                }
                const int p = pc[3];
                const double st = tp[(R.ST + gi) * LANES];
                double x;
                int pw = p;
                if (p > 0) {
                    x = (st * (2.0 - X) + Y) / X;
                } else {
                    x = Y / X;
                    pw = -p;
                }
                Gk = gpow<double>(Gk, x, pw);
                const double rX = 1.0 / X;
                const double along = p > 0 ? st + x : x;   // -(dx'/dB') * B'
                tp[(R.DXDV + gi) * LANES] = rX * dfdv * (sY - along * sX);
                tp[(R.DXDST + gi) * LANES] = p > 0 ? (2.0 - X) * rX : 0.0;
                const int j = gi - cg0;
                if (j < ADJ_MAX_GATES) {
                    gx[j] = x;
                    gp[j] = pw;
                } else if (v.status) {
                    atomicOr(v.status, ST_BAD_OP);
                }
                ++gi;
                pc += 5;
            } else if (code == M_ADDCURR) {
                sumg += Gk;
                ichan += Ek * Gk;
                const int ng = min(gi - cg0, ADJ_MAX_GATES);
                double prod = 1.0;
                for (int g = 0; g < ng; ++g) prod = gpow<double>(prod, gx[g], gp[g]);
                tp[(R.PROD + ci) * LANES] = prod;
                for (int g = 0; g < ng; ++g) {
                    double q = (double)gp[g];
                    for (int e = 1; e < gp[g]; ++e) q *= gx[g];
                    for (int h = 0; h < ng; ++h)
                        if (h != g) q = gpow<double>(q, gx[h], gp[h]);
                    tp[(R.Q + cg0 + g) * LANES] = q;
                }
                pc += 2;
            } else if (code == M_END) {
                const double tbyc = P[pc[1] * LANES];
                Rc[s * LANES] = Vm + ichan * tbyc;
                Dc[s * LANES] = sumg * tbyc + P[pc[2] * LANES];
                tp[(R.ICH + s) * LANES] = ichan;
                tp[(R.SG + s) * LANES] = sumg;
                pc += 4;
                break;
            } else {
                if (v.status) atomicOr(v.status, ST_BAD_OP);
                return;
            }
        }
    }
    for (int s = 0; s < S; ++s) {
        const int p = par[s * LANES];
        const double d = Dc[s * LANES];
        tp[(R.RD + s) * LANES] = 1.0 / d;
        tp[(R.RP + s) * LANES] = Rc[s * LANES];
        double temp = 0.0;
        if (p >= 0) {
            temp = Aw[s * LANES] / d;
            Dc[p * LANES] -= Bw[s * LANES] * temp;
            Rc[p * LANES] -= Rc[s * LANES] * temp;
        }
        tp[(R.T + s) * LANES] = temp;
    }
    for (int s = S - 1; s >= 0; --s) {
        const int p = par[s * LANES];
        double r = Rc[s * LANES];
        if (p >= 0) r -= Cw[s * LANES] * Rc[p * LANES];
        r = r / Dc[s * LANES];
        Rc[s * LANES] = r;
        tp[(R.X + s) * LANES] = r;
    }
}

// ---------------------------------------------------------------- reverse
// grid (tiles), ADJ_REV_WARPS warps per tile. Warp 0 runs the elimination's
// reverse (a chain along the tree); the channel phase and the seeds of the
// next step are split over the warps by slot (slot s to warp s mod W), so
// the block keeps every FP64 unit of its SM busy. Shared memory: the D and R
// adjoint columns (2 * smax * 32 doubles), per-warp loss partials
// (W * 32 doubles) and the tile type's slot and channel plans.
constexpr int ADJ_REV_WARPS = 4;

__global__ void __launch_bounds__(ADJ_REV_WARPS * 32)
k_adj_reverse(AdjView v, int smax, int hmax, int nk, int step0)
{
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    const int t = blockIdx.x;
    const Tile tl = v.tiles[t];
    const TileType ty = v.types[tl.type];
    const AdjType at = v.atypes[tl.type];
    const int S = at.nslots;
    const bool crank = ty.crank != 0;
    const AdjRows R = adj_rows(S, at.ngates, at.nchans);
    const double *P = v.P + tl.fld * LANES + lane;
    const int *par = v.parent + tl.topo * LANES + lane;
    const double *Bw = v.B + tl.topo * LANES + lane;
    const double *Cw = v.Cb + tl.topo * LANES + lane;
    const int *tgt = v.tgt + tl.topo * LANES + lane;
    double *Vb = v.Vbar + tl.vm * LANES + lane;
    double *Xb = v.Xbar + v.xb_off[t] * LANES + lane;
    double *loss = v.loss + (size_t)t * LANES + lane;
    double *Db = sm + lane;
    double *Rb = Db + (size_t)smax * LANES;
    double *lpart = sm + (size_t)2 * smax * LANES;       // [warp][lane]
    AdjSlot *slots = reinterpret_cast<AdjSlot *>(lpart + nw * LANES);
    AdjChan *chans = reinterpret_cast<AdjChan *>(slots + smax);
    for (int i = threadIdx.x; i < S; i += blockDim.x) slots[i] = v.slot_plan[at.slot_off + i];
    for (int i = threadIdx.x; i < at.nchans && i < hmax; i += blockDim.x) chans[i] = v.chan_plan[at.chan_off + i];

    // seed of step k at slot s: vb is the adjoint of Vm after step k
    auto seed = [&](int k, int s, double vb) {
        double l = 0.0;
        const int j = tgt[s * LANES];
        if (j >= 0) {
            const double *tp = adj_tape(v, k, t, lane);
            const double x = __ldg(tp + (R.X + s) * LANES);
            const double vnext = crank ? x + x - __ldg(tp + (R.V + s) * LANES) : x;
            const double diff = vnext - __ldg(v.trace + (size_t)(step0 + k) * v.ntargets + j);
            l = diff * diff;
            vb += 2.0 * diff;
        }
        Rb[s * LANES] = crank ? 2.0 * vb : vb;
        Vb[s * LANES] = crank ? -vb : 0.0;
        return l;
    };

    double lw = 0.0;
    for (int s = warp; s < S; s += nw) lw += seed(nk - 1, s, Vb[s * LANES]);
    lpart[warp * LANES + lane] = lw;
    __syncthreads();
    for (int k = nk - 1; k >= 0; --k) {
        double *tp = adj_tape(v, k, t, lane);
        if (warp == 0) {
            // loss of step k, summed in warp order, steps descending
            double l = 0.0;
            for (int w = 0; w < nw; ++w) l += lpart[w * LANES + lane];
            *loss += l;
            // back substitution reversed
#pragma unroll 4
            for (int s = 0; s < S; ++s) {
                const int p = __ldg(par + s * LANES);
                const double rb = Rb[s * LANES] * __ldg(tp + (R.RD + s) * LANES);
                Rb[s * LANES] = rb;
                tp[(R.RBBS + s) * LANES] = rb;
                if (p >= 0) Rb[p * LANES] -= __ldg(Cw + s * LANES) * rb;
                Db[s * LANES] = -__ldg(tp + (R.X + s) * LANES) * rb;
            }
            // forward elimination reversed
#pragma unroll 4
            for (int s = S - 1; s >= 0; --s) {
                const int p = __ldg(par + s * LANES);
                if (p < 0) continue;
                const double tt = __ldg(tp + (R.T + s) * LANES);
                const double rd = __ldg(tp + (R.RD + s) * LANES);
                const double tb = -__ldg(Bw + s * LANES) * Db[p * LANES] - __ldg(tp + (R.RP + s) * LANES) * Rb[p * LANES];
                Rb[s * LANES] -= tt * Rb[p * LANES];
                Db[s * LANES] -= tt * (tb * rd);
            }
        }
        __syncthreads();
        // channels reversed (adjoint of Vm and of the gate states), then the
        // seed of step k-1
        lw = 0.0;
        for (int s = warp; s < S; s += nw) {
            const AdjSlot sp = slots[s];
            const double rb = Rb[s * LANES], db = Db[s * LANES];
            tp[(R.RBF + s) * LANES] = rb;
            tp[(R.DBF + s) * LANES] = db;
            const double tbyc = __ldg(P + sp.f_tbyc * LANES);
            const double Ibar = rb * tbyc, Sbar = db * tbyc;
            double vbn = Vb[s * LANES] + rb;
            for (int c = sp.ch0; c < sp.ch0 + sp.nch; ++c) {
                const AdjChan ch = c < hmax ? chans[c] : v.chan_plan[at.chan_off + c];
                const double Ek = ch.f_ek >= 0 ? __ldg(P + ch.f_ek * LANES) : 0.0;
                const double w = (Sbar + Ibar * Ek) * __ldg(P + ch.f_gmax * LANES);
#pragma unroll 2
                for (int g = ch.g0; g < ch.g0 + ch.ng; ++g) {
                    const double xhat = Xb[g * LANES] + w * __ldg(tp + (R.Q + g) * LANES);
                    vbn += xhat * __ldg(tp + (R.DXDV + g) * LANES);
                    Xb[g * LANES] = xhat * __ldg(tp + (R.DXDST + g) * LANES);
                }
            }
            if (k > 0) lw += seed(k - 1, s, vbn);
            else Vb[s * LANES] = vbn;
        }
        lpart[warp * LANES + lane] = lw;
        __syncthreads();
    }
}

// ---------------------------------------------------------------- gradient sums
// grid (tiles, smax), 32 threads: one (tile, slot) per block, one lane per
// thread. Sums the segment's steps in descending order onto the totals.
__global__ void __launch_bounds__(32)
k_adj_reduce(AdjView v, int nk)
{
    const int lane = threadIdx.x;
    const int t = blockIdx.x;
    const int s = blockIdx.y;
    const Tile tl = v.tiles[t];
    const AdjType at = v.atypes[tl.type];
    if (s >= at.nslots) return;
    const AdjRows R = adj_rows(at.nslots, at.ngates, at.nchans);
    const AdjSlot sp = v.slot_plan[at.slot_off + s];
    const double *P = v.P + tl.fld * LANES + lane;
    double *Gf = v.Gf + tl.fld * LANES + lane;
    const int64_t topo = (tl.topo + s) * LANES + lane;
    const int p = v.parent[topo];
    const double tbyc = P[sp.f_tbyc * LANES];
    double g_i = Gf[sp.f_emrm * LANES];     // Em/Rm and inject share the adjoint of ichan
    double g_j = Gf[sp.f_inj * LANES];
    double g_t = Gf[sp.f_tbyc * LANES];
    double g_d = Gf[sp.f_diag * LANES];
    double ga = v.GA[topo], gb = v.GB[topo], gc = v.GC[topo];
    const double B = v.B[topo];
    for (int k = nk - 1; k >= 0; --k) {
        const double *tp = adj_tape(v, k, t, lane);
        const double rb = tp[(R.RBF + s) * LANES], db = tp[(R.DBF + s) * LANES];
        const double ib = rb * tbyc;
        g_i += ib;
        g_j += ib;
        g_t += rb * tp[(R.ICH + s) * LANES] + db * tp[(R.SG + s) * LANES];
        g_d += db;
        if (p >= 0) {
            gc -= tp[(R.X + p) * LANES] * tp[(R.RBBS + s) * LANES];
            const double dbp = tp[(R.DBF + p) * LANES], rbp = tp[(R.RBF + p) * LANES];
            gb -= tp[(R.T + s) * LANES] * dbp;
            ga += (-B * dbp - tp[(R.RP + s) * LANES] * rbp) * tp[(R.RD + s) * LANES];
        }
    }
    Gf[sp.f_emrm * LANES] = g_i;
    Gf[sp.f_inj * LANES] = g_j;
    Gf[sp.f_tbyc * LANES] = g_t;
    Gf[sp.f_diag * LANES] = g_d;
    v.GA[topo] = ga;
    v.GB[topo] = gb;
    v.GC[topo] = gc;
    // channels of the slot: Ek and gmax gradients, kept per channel
    for (int c = sp.ch0; c < sp.ch0 + sp.nch; ++c) {
        const AdjChan ch = v.chan_plan[at.chan_off + c];
        const double Ek = ch.f_ek >= 0 ? P[ch.f_ek * LANES] : 0.0;
        const double gmax = P[ch.f_gmax * LANES];
        double *gek = v.Gek + (v.ch_off[t] + c) * LANES + lane;
        double *ggm = v.Ggm + (v.ch_off[t] + c) * LANES + lane;
        double a = *gek, b = *ggm;
        for (int k = nk - 1; k >= 0; --k) {
            const double *tp = adj_tape(v, k, t, lane);
            const double ib = tp[(R.RBF + s) * LANES] * tbyc, sb = tp[(R.DBF + s) * LANES] * tbyc;
            const double prod = tp[(R.PROD + c) * LANES];
            a += ib * gmax * prod;
            b += (sb + ib * Ek) * prod;
        }
        *gek = a;
        *ggm = b;
    }
}

}  // namespace gbh
