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
#include "gbh_internal.h"
#include "gbh_devfn.cuh"

namespace gbh {

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

    for (int it = 0; it < nsteps; ++it) {
        const long long step = sbase + step0 + it;
        VCursor vc, cc;
        if (tg.ncols) { vc.lo = vc.hi = 0.0; } else { vc.lo = -1e20; vc.hi = 1e20; }
        vc.row = vc.base = 0; vc.frac = 0.0;
        cc.lo = cc.hi = 0.0; cc.row = cc.base = 0; cc.frac = 0.0;
        double save_frac = 0.0;
        int tab_base = 0, ctab_base = 0, sel = 0;
        double Ek = 0.0, Gk = 0.0, gmax = 0.0, Ik = 0.0, GHK = 0.0;
        int doGHK = 0;

        // ---------------- channel phase ----------------
        const int *pc = v.prog + ty.prog_off;
        for (int s = 0; s < S; ++s) {
            const double Vm = Vw[s * LANES];
            double sumg = 0.0, ichan = 0.0, Im = 0.0;
            for (;;) {
                const int code = pc[0];
                if (code == M_BEGIN) {
                    const double emrm = Pw[pc[1] * LANES];
                    ichan = emrm + Pw[pc[2] * LANES];
                    if (GIV) {
                        Im = emrm - Vm / Pw[pc[3] * LANES];
                        Gw[pc[4] * LANES] = Im;
                    }
                    pc += 5;
                } else if (code == M_NEWVOLT) {
                    locate(vc, Vm, tg.xmin, tg.invdx, tg.xdivs, xvals, ncols, interp);
                    pc += 1;
                } else if (code == M_CONCVAL) {
                    sel = pc[1];
                    Fw[sel * LANES] = 0.0;
                    pc += 2;
                } else if (code == M_DOMAIN) {
                    const double concen = Pw[pc[1] * LANES] * Ik;
                    locate(cc, concen, tg.ymin, tg.invdy, tg.ydivs, yvals, ncols, interp);
                    ctab_base = cc.base;
                    pc += 2;
                } else if (code == M_NEWCONC2) {
                    const double concen = Cw[pc[1] * LANES];
                    tab_base = ctab_base;
                    save_frac = cc.frac;
                    locate(cc, concen, tg.ymin, tg.invdy, tg.ydivs, yvals, ncols, interp);
                    ctab_base = cc.base;
                    pc += 2;
                } else if (code == M_NEWCONC1) {
                    const double concen = Cw[sel * LANES];
                    locate(cc, concen, tg.ymin, tg.invdy, tg.ydivs, yvals, ncols, interp);
                    ctab_base = cc.base;
                    pc += 1;
                } else if (code == M_SPIKE) {
                    int cnt = Iw[pc[2] * LANES] - 1;
                    if (Vm > Pw[pc[1] * LANES]) {
                        if (cnt <= 0 && active) {
                            // h_dospike_event: deliver to every target synchan
                            const int64_t e0 = v.syn_out_start[neuron], e1 = v.syn_out_start[neuron + 1];
                            for (int64_t e = e0; e < e1; ++e) {
                                const int slot = (int)((step + v.syn_out_delay[e]) % v.ring_len);
                                atomicAdd(&v.ring[v.syn_out_base[e] + (int64_t)slot * LANES], 1u);
                            }
                            v.spikes[neuron] += 1ULL;
                            if (v.spiked) atomicOr(&v.spiked[neuron >> 5], 1u << (neuron & 31));
                            cnt = Iw[pc[3] * LANES];
                        }
                    }
                    Iw[pc[2] * LANES] = cnt;
                    pc += 4;
                } else if (code == M_ELMMPUMP) {
                    const double cx = Cw[sel * LANES];
                    const double X = 1.0 / (cx + Pw[pc[1] * LANES]);
                    const double vmax = Pw[pc[2] * LANES];
                    ichan += Ik = vmax * cx * X;
                    if (GIV) Gw[pc[4] * LANES] = c5 ? Ik / vmax : Ik;
                    Im += Ik;
                    if (ty.has_cd) v.CD[(tl.pools + sel) * LANES + lane] += Pw[pc[3] * LANES] * X;   // hines_chip.c:301
                    pc += 5;
                } else if (code == M_FLUX) {
                    Fw[sel * LANES] += Ik;
                    pc += 1;
                } else if (code == M_SCALE_FLUX) {
                    Fw[sel * LANES] += Pw[pc[1] * LANES] * Ik;
                    pc += 2;
                } else if (code == M_STORE) {
                    pc += 3;  // itotal accumulation is host-visible only; rejected at setup
                } else if (code == M_END) {
                    const double tbyc = Pw[pc[1] * LANES];
                    Rcol[s * LANES] = Vm + ichan * tbyc;
                    Dcol[s * LANES] = sumg * tbyc + Pw[pc[2] * LANES];
                    if (GIV) Gw[pc[3] * LANES] = Im;
                    pc += 4;
                    break;
                } else {
                    // current-producing ops, then the conductance sub-program
                    bool current = true;
                    if (code == M_GHK) {
                        const double cin = Cw[sel * LANES], cout = Cw[(sel + 1) * LANES];
                        GHK = Pw[pc[1] * LANES];
                        double X = Vm * GHK;
                        double Y = exp(-X);
                        Ek = Pw[pc[2] * LANES];
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
                        gmax = Pw[pc[3] * LANES];
                        Gk = gmax * GHK;
                        pc += 4;
                    } else if (code == M_SAME_GHK) {
                        gmax = Pw[pc[1] * LANES];
                        Gk = gmax * GHK;
                        pc += 2;
                    } else if (code == M_DO_TABGHK) {
                        doGHK = 1;
                        pc += 1;
                    } else if (code == M_NERNST) {
                        Ek = log(Cw[(sel + 1) * LANES] / Cw[sel * LANES]) * Pw[pc[1] * LANES];
                        gmax = Gk = Pw[pc[2] * LANES];
                        pc += 3;
                    } else if (code == M_CHAN) {
                        Ek = Pw[pc[1] * LANES];
                        gmax = Gk = Pw[pc[2] * LANES];
                        pc += 3;
                    } else if (code == M_CHAN_G) {
                        gmax = Gk = Pw[pc[1] * LANES];
                        pc += 2;
                    } else {
                        current = false;
                        if (v.status) atomicOr(v.status, ST_BAD_OP);
                        return;
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
                                double *st = &Pw[pc[4] * LANES];
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
                            double *px = &Pw[pc[4] * LANES];
                            double *py = &Pw[pc[5] * LANES];
                            if (pc[1] >= 0) {
                                const uint64_t key = ((uint64_t)neuron << 24) ^ ((uint64_t)step << 1) ^
                                                     (uint64_t)pc[4];
                                if (syn3_uniform(key) <= Pw[pc[1] * LANES]) *px += sl[3];
                            }
                            double X = *px * sl[0];
                            unsigned *cell = v.ring + ((tl.syn + (int64_t)pc[3] * v.ring_len +
                                                        (int64_t)(step % v.ring_len)) * LANES + lane);
                            const unsigned n = *cell;
                            if (n) {
                                const double wdt = Pw[pc[6] * LANES];
                                double act = 0.0;
                                for (unsigned q = 0; q < n; ++q) act += wdt;
                                X += v.dt * act * sl[3];
                                *cell = 0u;
                            }
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
                                    Gw[g * LANES] = Gk / gmax;
                                    Gw[(g + 1) * LANES] = Gk * (Ek - Vm) / gmax;
                                } else {
                                    Gw[g * LANES] = Gk;
                                    Gw[(g + 1) * LANES] = Gk * (Ek - Vm);
                                }
                                Gw[(g + 2) * LANES] = Ek;
                            }
                            const double X = Pw[pc[1] * LANES] * exp(Vm * Pw[pc[2] * LANES]);
                            Gk *= X / (X + Pw[pc[3] * LANES]);
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
                                    Gw[g * LANES] = Gk / gmax;
                                    Gw[(g + 1) * LANES] = Ik / gmax;
                                } else {
                                    Gw[g * LANES] = Gk;
                                    Gw[(g + 1) * LANES] = Ik;
                                }
                                Gw[(g + 2) * LANES] = Ek;
                            }
                            pc += 2;
                        } else {
                            if (v.status) atomicOr(v.status, ST_BAD_OP);
                            return;
                        }
                        Im += Ik;
                        break;
                    }
                }
            }
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
            if (!pool_phase(v.prog + ty.pool_off, PL)) {
                if (v.status) atomicOr(v.status, ST_BAD_OP);
                return;
            }
        }

        // ---------------- elimination ----------------
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
        // cooperative multi-step launch: every tile's events of this step
        // are in the rings before any tile starts the next step
        if (v.gbar && !grid_sync(v.gbar, gridDim.x, v.status)) return;
    }
}

// Launchers, one per precision translation unit (the FP64 unit is compiled
// without multiply-add contraction, the mixed unit with it).
cudaError_t launch_fp64(const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                        long long step, bool giv, cudaStream_t st);
cudaError_t launch_mixed(const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                         long long step, bool giv, cudaStream_t st);

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
