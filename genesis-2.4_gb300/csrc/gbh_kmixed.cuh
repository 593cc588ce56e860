// gbh_kmixed.cuh -- the mixed-precision step kernel.
//
// Same tile layout and decoded programs as k_steps (gbh_kernels.cuh), with
//   * gate and table arithmetic -- table interpolation, the trapezoid /
//     instantaneous gate update, gate powers, conductance and current sums --
//     in double-float on FP32 instructions (gbh_df.cuh), tables stored as
//     (value, next-row difference) double-float pairs;
//   * Vm, the rhs/diagonal of each row, the Hines elimination and the Ca pools
//     in FP64, the elimination dividing through a reciprocal refined by one
//     Newton step from an FP32 seed (one reciprocal per row instead of two
//     IEEE divisions);
//   * conversions between the two representations on the integer pipe.
// It does not reproduce the reference bit for bit; its error against the
// FP64 CPU solver is measured and reported instead.
#pragma once
#include "gbh_df.cuh"
#include "gbh_kernels.cuh"

namespace gbh {


// Per-type constants of the mixed compartment interpreter.
struct ChanEnvDF {
    const float4 *tab;
    TableGeom tg;
    int ncols;
    df xnmin, xinv, ynmin, yinv;
    bool c5, has_cd;
};

// Carried state of the mixed interpreter (reset every step).
struct ChanStateDF {
    DCursor vc, cc, c1;
    int sel;
    df Ek, Gk, gmax;
    double GHK, Ik;
    int doGHK;
};

__device__ __forceinline__ void chan_state_reset_df(ChanStateDF &cs)
{
    cs.vc.row = cs.vc.base = 0;
    cs.vc.frac = df_make(0.f, 0.f);
    cs.cc = cs.vc;
    cs.c1 = cs.vc;
    cs.sel = 0;
    cs.Ek = cs.Gk = cs.gmax = df_make(0.f, 0.f);
    cs.GHK = cs.Ik = 0.0;
    cs.doGHK = 0;
}

// One compartment of the mixed form: double-float gates, FP64 row terms.
template <bool GIV, int STR>
__device__ __forceinline__ bool chan_compartment_df(const DevView &v, const ChanEnvDF &E, ChanStateDF &cs,
                                                    const ChanRows &N, const int *&pc, double Vm, long long step,
                                                    double &R, double &D)
{
    DCursor &vc = cs.vc, &cc = cs.cc, &c1 = cs.c1;
    int &sel = cs.sel;
    df &Ek = cs.Ek, &Gk = cs.Gk, &gmax = cs.gmax;
    double &GHK = cs.GHK, &Ik = cs.Ik;
    int &doGHK = cs.doGHK;
    const float4 *tab = E.tab;
    const TableGeom &tg = E.tg;
    const int ncols = E.ncols;
    const df xnmin = E.xnmin, xinv = E.xinv, ynmin = E.ynmin, yinv = E.yinv;
    const bool c5 = E.c5;
    const int64_t neuron = N.neuron;
    const bool active = N.active;
    (void)neuron;
    (void)active;
    (void)c1;
    const df vmd = d2df(Vm);
    df sumg = df_make(0.f, 0.f), ichan = sumg;
    double Im = 0.0;
    for (;;) {

        const int code = pc[0];
        if (code == M_BEGIN) {
            const df emrm = ld_df(&N.P[(pc[1]) * STR]);
            ichan = df_add(emrm, ld_df(&N.P[(pc[2]) * STR]));
            if (GIV) {
                Im = df2d(emrm) - Vm / N.P[(pc[3]) * STR];
                N.G[(pc[4]) * STR] = Im;
            }
            pc += 5;
        } else if (code == M_NEWVOLT) {
            locate_df(vc, vmd, xnmin, xinv, tg.xdivs, ncols);
            pc += 1;
        } else if (code == M_CONCVAL) {
            sel = pc[1];
            N.F[(sel) * STR] = 0.0;
            pc += 2;
        } else if (code == M_DOMAIN) {
            locate_df(cc, d2df(N.P[(pc[1]) * STR] * Ik), ynmin, yinv, tg.ydivs, ncols);
            pc += 2;
        } else if (code == M_NEWCONC2) {
            c1 = cc;
            locate_df(cc, d2df(N.C[(pc[1]) * STR]), ynmin, yinv, tg.ydivs, ncols);
            pc += 2;
        } else if (code == M_NEWCONC1) {
            locate_df(cc, d2df(N.C[(sel) * STR]), ynmin, yinv, tg.ydivs, ncols);
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
            Ik = vmax * cx * X;
            ichan = df_add(ichan, d2df(Ik));
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
            N.IT[pc[2] * STR] += pc[1] ? df2d(Gk) : Ik;
            pc += 3;
        } else if (code == M_ITLEAK) {
            N.IT[pc[3] * STR] += df2d(ld_df(&N.P[(pc[1]) * STR])) - Vm / N.P[(pc[2]) * STR];
            pc += 4;
        } else if (code == M_END) {
            const df tbyc = ld_df(&N.P[(pc[1]) * STR]);
            const df dv = df_mul(ichan, tbyc);
            R = df2d(df_add(vmd, dv));
            D = df2d(df_add(df_mul(sumg, tbyc), ld_df(&N.P[(pc[2]) * STR])));
            if (GIV) N.G[(pc[3]) * STR] = Im;
            pc += 4;
            break;
        } else {
            if (code == M_GHK) {
                const double cin = N.C[(sel) * STR], cout = N.C[((sel + 1)) * STR];
                double g = N.P[(pc[1]) * STR];
                const double X = Vm * g;
                const double Y = exp(-X);
                double e = N.P[(pc[2]) * STR];
                double ik = e * (cin - (Y * cout));
                double gk;
                if (fabs(X) < 1.0e-6) {
                    gk = 1.0 - 0.5 * X;
                    g = 0.5 * g * e * (cin + cout);
                    ik = -ik / gk;
                } else {
                    gk = 1.0 - Y;
                    g = g * (ik / gk - e * g * (cin - cout) * Vm * Y / (gk * gk));
                    ik = -X * ik / gk;
                }
                GHK = g;
                Ek = d2df((ik + g * Vm) / g);
                gmax = d2df(N.P[(pc[3]) * STR]);
                Gk = d2df(N.P[(pc[3]) * STR] * GHK);
                pc += 4;
            } else if (code == M_SAME_GHK) {
                gmax = d2df(N.P[(pc[1]) * STR]);
                Gk = d2df(N.P[(pc[1]) * STR] * GHK);
                pc += 2;
            } else if (code == M_DO_TABGHK) {
                doGHK = 1;
                pc += 1;
            } else if (code == M_NERNST) {
                Ek = d2df(log(N.C[((sel + 1)) * STR] / N.C[(sel) * STR]) * N.P[(pc[1]) * STR]);
                gmax = Gk = d2df(N.P[(pc[2]) * STR]);
                pc += 3;
            } else if (code == M_CHAN) {
                Ek = ld_df(&N.P[(pc[1]) * STR]);
                gmax = Gk = ld_df(&N.P[(pc[2]) * STR]);
                pc += 3;
            } else if (code == M_CHAN_G) {
                gmax = Gk = ld_df(&N.P[(pc[1]) * STR]);
                pc += 2;
            } else {
                if (v.status) atomicOr(v.status, ST_BAD_OP);
                return false;
            }
            for (;;) {
                const int k = pc[0];
                if (k == M_GATE) {
                    const int kind = pc[1];
                    df X, Y;
                    if (kind == GK_1V || kind == GK_1C) {
                        const DCursor &cu = (kind == GK_1V) ? vc : cc;
                        const int b = cu.base + pc[2];
                        X = interp_df(tab, b, cu.frac);
                        Y = interp_df(tab, b + 1, cu.frac);
                    } else {
                        // 2-D tables: rows from the voltage (or first conc) cursor,
                        // columns from the conc cursor
                        const DCursor &ru = (kind == GK_2V) ? vc : c1;
                        const int b = ru.base + cc.row + cc.row + pc[2];
                        const df cf = cc.frac, rf = ru.frac;
                        const df one_c = df_add_f(df_neg(cf), 1.0f), one_r = df_add_f(df_neg(rf), 1.0f);
                        df q[2];
                        for (int h = 0; h < 2; ++h) {
                            const df t00 = val_df(tab, b + h), t01 = val_df(tab, b + 2 + h);
                            const df t10 = interp_df(tab, b + h, df_make(1.f, 0.f));
                            const df t11 = interp_df(tab, b + 2 + h, df_make(1.f, 0.f));
                            const df lo = df_add(df_mul(one_c, t00), df_mul(cf, t01));
                            const df hi = df_add(df_mul(one_c, t10), df_mul(cf, t11));
                            q[h] = df_add(df_mul(one_r, lo), df_mul(rf, hi));
                        }
                        X = q[0];
                        Y = q[1];
                    }
                    const int p = pc[3];
                    if (p == 0) {
                        Ek = Y;
                        pc += 5;
                        if (doGHK) {
                            GHK = df2d(X);
                            doGHK = 0;
                            break;
                        }
                        Gk = df_mul(Gk, X);
                        continue;
                    }
                    double *st = &N.P[(pc[4]) * STR];
                    df x;
                    int pw = p;
                    if (p > 0) {
                        x = df_div(df_add(df_mul(ld_df(st), df_add_f(df_neg(X), 2.0f)), Y), X);
                    } else {
                        x = df_div(Y, X);
                        pw = -p;
                    }
                    st_df(st, x);
                    Gk = dpow(Gk, x, pw);
                    pc += 5;
                    continue;
                } else if (k == M_SYN) {
                    const double *sl = v.stablist + pc[2];
                    double *px = &N.P[(pc[4]) * STR];
                    double *py = &N.P[(pc[5]) * STR];
                    if (pc[1] >= 0) {
                        const uint64_t key = ((uint64_t)neuron << 24) ^ ((uint64_t)step << 1) ^
                                             (uint64_t)pc[4];
                        if (syn3_uniform(key) <= N.P[(pc[1]) * STR]) *px += sl[3];
                    }
                    double X = *px * sl[0];
                    unsigned *cell = N.ring + ((int64_t)pc[3] * v.ring_len + (int64_t)(step % v.ring_len)) * LANES;
                    double act;
                    if (syn_due(v, cell, N.P[(pc[6]) * STR], step, act)) X += v.dt * act * sl[3];
                    *px = X;
                    const double Y = X * sl[1] + *py * sl[2];
                    *py = Y;
                    Gk = df_mul(Gk, d2df(Y));
                    pc += 7;
                    continue;
                } else if (k == M_MGBLOCK) {
                    const double gk = df2d(Gk), ek = df2d(Ek);
                    if (GIV) {
                        const int g = pc[4];
                        const double gm = c5 ? df2d(gmax) : 1.0;
                        N.G[(g) * STR] = gk / gm;
                        N.G[((g + 1)) * STR] = gk * (ek - Vm) / gm;
                        N.G[((g + 2)) * STR] = ek;
                    }
                    const double X = N.P[(pc[1]) * STR] * exp(Vm * N.P[(pc[2]) * STR]);
                    Gk = d2df(gk * (X / (X + N.P[(pc[3]) * STR])));
                    pc += 5;
                    continue;
                } else if (k == M_ADDCURR) {
                    const int g = pc[1];
                    sumg = df_add(sumg, Gk);
                    ichan = df_add(ichan, df_mul(Ek, Gk));
                    const double gk = df2d(Gk), ek = df2d(Ek);
                    Ik = gk * (ek - Vm);
                    if (GIV) {
                        const double gm = c5 ? df2d(gmax) : 1.0;
                        N.G[(g) * STR] = gk / gm;
                        N.G[((g + 1)) * STR] = Ik / gm;
                        N.G[((g + 2)) * STR] = ek;
                    }
                    Im += Ik;
                    pc += 2;
                    break;
                } else {
                    if (v.status) atomicOr(v.status, ST_BAD_OP);
                    return false;
                }
            }
        }
    }
    return true;
}

template <bool GIV>
__global__ void __launch_bounds__(128, 6)
k_steps_mixed(DevView v, int tile0, int tile1, int smax, int nsteps, long long step0)
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
    const float4 *tab = v.tabdf + tg.tab_off;
    const int ncols = tg.ncols;
    const df xnmin = df_make(-tg.xmin_hi, -tg.xmin_lo), xinv = df_make(tg.invdx_hi, tg.invdx_lo);
    const df ynmin = df_make(-tg.ymin_hi, -tg.ymin_lo), yinv = df_make(tg.invdy_hi, tg.invdy_lo);
    const bool c5 = ty.chanmode5 != 0;
    const bool active = lane < tl.nlanes;

    double *Pw = v.P + tl.fld * LANES + lane;
    int *Iw = v.I + tl.ints * LANES + lane;
    double *Vw = v.V + tl.vm * LANES + lane;
    double *Cw = v.C + tl.pools * LANES + lane;
    double *Fw = v.F + tl.pools * LANES + lane;
    double *Gw = v.giv + tl.giv * LANES + lane;
    const int *par = v.parent + tl.topo * LANES + lane;
    const double *Aw = v.A + tl.topo * LANES + lane;
    const double *Bw = v.B + tl.topo * LANES + lane;
    const double *Cbw = v.Cb + tl.topo * LANES + lane;
    double *Dcol = sm + (size_t)wib * 2 * smax * LANES + lane;   // diagonal, then its reciprocal
    double *Rcol = Dcol + (size_t)smax * LANES;
    const int S = ty.nslots;
    const int64_t neuron = tl.first_neuron + lane;

    ChanEnvDF E;
    E.tab = tab;
    E.tg = tg;
    E.ncols = ncols;
    E.xnmin = xnmin;
    E.xinv = xinv;
    E.ynmin = ynmin;
    E.yinv = yinv;
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
        ChanStateDF cs;
        chan_state_reset_df(cs);
        const int *pc = v.prog + ty.prog_off;
        for (int s = 0; s < S; ++s) {
            double R, D;
            if (!chan_compartment_df<GIV, LANES>(v, E, cs, NR, pc, Vw[s * LANES], step, R, D)) {
                if (v.status) atomicOr(v.status, ST_BAD_OP);
                return;
            }
            Rcol[s * LANES] = R;
            Dcol[s * LANES] = D;
        }

        // Ca pools (FP64)
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

        // elimination (FP64, one refined reciprocal per row; symmetric
        // compartments: the reference's program with its divisions)
        if (ty.sym) {
            sym_eliminate<LANES>(v.prog + ty.sym_off, Rcol, Dcol, v.RV + tl.rav * LANES + lane, Vw, ty.crank != 0);
        } else {
        for (int s = 0; s < S; ++s) {
            const int p = par[s * LANES];
            const double ri = rcp_newton(Dcol[s * LANES]);
            Dcol[s * LANES] = ri;   // the row's diagonal is final here; keep only its reciprocal
            if (p >= 0) {
                const double temp = Aw[s * LANES] * ri;
                Dcol[p * LANES] = fma(-Bw[s * LANES], temp, Dcol[p * LANES]);
                Rcol[p * LANES] = fma(-Rcol[s * LANES], temp, Rcol[p * LANES]);
            }
        }
        for (int s = S - 1; s >= 0; --s) {
            const int p = par[s * LANES];
            double r = Rcol[s * LANES];
            if (p >= 0) r = fma(-Cbw[s * LANES], Rcol[p * LANES], r);
            r = r * Dcol[s * LANES];
            Rcol[s * LANES] = r;
            if (ty.crank) {
                const double old = Vw[s * LANES];
                Vw[s * LANES] = fma(2.0, r, -old);
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

// Stack elimination of the mixed form (see k_stack in gbh_kernels.cuh): the
// same row order and per-lane stacks; the diagonal's reciprocal is formed
// once per row (rcp_newton) and kept in the column for back substitution.
//
// SPLIT: two warps per tile. After a launch's first step the second warp
// runs the channel phase of the rows above the static ones (kSplitRows at
// most; the soma of a tree whose dendrites are passive) and the pool phase,
// leaving each row's (R, D) in shared memory, while the first warp sweeps
// the static rows; the first warp then finishes those rows' forward steps
// and the back substitution. Both warps pass two barriers per step.
template <bool GIV, bool SPLIT>
__global__ void __launch_bounds__(SPLIT ? 64 : 32, SPLIT ? 8 : 16)
k_stack_mixed(DevView v, int tile0, int tile1, int cap, int nsteps, long long step0)
{
    extern __shared__ double sm[];
    __shared__ int sbad;
    const int lane = threadIdx.x & (LANES - 1);
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
    const int wid = SPLIT ? (int)(threadIdx.x >> 5) : 0;   // 0 sweeps, 1 computes the channel rows
    const long long sbase = v.step_dev ? *v.step_dev : 0;
    const Tile tl = v.tiles[t];
    const TileType ty = v.types[tl.type];
    const TableGeom tg = v.tgeom[ty.table_set];
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
    double *stk = sm + lane;
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

    ChanEnvDF E;
    E.tab = v.tabdf + tg.tab_off;
    E.tg = tg;
    E.ncols = tg.ncols;
    E.xnmin = df_make(-tg.xmin_hi, -tg.xmin_lo);
    E.xinv = df_make(tg.invdx_hi, tg.invdx_lo);
    E.ynmin = df_make(-tg.ymin_hi, -tg.ymin_lo);
    E.yinv = df_make(tg.invdy_hi, tg.invdy_lo);
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
        // factor) are in kst (see k_stack)
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
            ChanStateDF cs1;
            chan_state_reset_df(cs1);
            const int *pc1 = v.prog + ty.prog_off + 9 * nst;   // a passive row's program is 9 ints
            for (int s = nst; s < S && !bad; ++s) {
                double R, D;
                if (!chan_compartment_df<GIV, LANES>(v, E, cs1, NR, pc1, Vw[s * LANES], step, R, D)) {
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
        ChanStateDF cs;
        chan_state_reset_df(cs);
        const int *pc = v.prog + ty.prog_off;
        int top = 0;
        double cd = 0.0, cr = 0.0;
        // the forward step of row s from its own (R, D): children's
        // contributions (stack, then the carried last child), the row's
        // reciprocal into the column, its own contribution pushed or carried;
        // a static row also keeps its rhs term K and its factor a / D
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
            const double ri = rcp_newton(D);
            col[s * LANES] = make_double2(R, ri);
            double temp = 0.0;
            if (f & FL_PARENT) {
                temp = a * ri;
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
            if (s < nst) kst[s * LANES] = make_double2(K, temp);
        };
        // a static row on later steps: only its rhs is eliminated; its
        // diagonal contribution is formed only for a parent above the static rows
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
                    if (f & FL_PD) cd = __ldg(&Bw[s * LANES]) * T;
                } else {
                    if (f & FL_PD) stk[(2 * top) * LANES] = __ldg(&Bw[s * LANES]) * T;
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
            R = (f & FL_CARRY_IN) ? R - cr : R;   // the carried child first: the stacked one's
            R = pop ? R - sv : R;                  // shared-memory load overlaps that subtraction
            reinterpret_cast<double *>(col + s * LANES)[0] = R;
            const double pr = R * T;
            if (f & FL_PD) {   // a parent above the static rows: its diagonal contribution
                const double pd = __ldg(&Bw[s * LANES]) * T;
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
            R = (f & FL_CARRY_IN) ? R - cr : R;   // (as in fwd_static1)
            R = (f & 1) ? R - sv : R;
            reinterpret_cast<double *>(col + s * LANES)[0] = R;
            const double pr = R * T;
            if (f & FL_PD) {   // a parent above the static rows: its diagonal contribution
                const double pd = __ldg(&Bw[s * LANES]) * T;
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
            const df ichan = df_add(ld_df(&Pw[ps[2] * LANES]), ld_df(&Pw[ps[3] * LANES]));
            const double K = df2d(df_mul(ichan, ld_df(&Pw[ps[4] * LANES])));
            kst[s * LANES].x = K;
            return K;
        };
        // a passive row (M_BEGIN / M_END): its current term ichan * tbyc in
        // double-float, added to Vm in FP64 (part of the Vm update); the
        // diagonal is the row's diagonal term (its conductance sum is zero)
        auto passive = [&](int s, const int *ps, double &R, double &D, double &K) {
            const df ichan = df_add(ld_df(&Pw[ps[2] * LANES]), ld_df(&Pw[ps[3] * LANES]));
            K = df2d(df_mul(ichan, ld_df(&Pw[ps[4] * LANES])));
            R = Vw[s * LANES] + K;
            D = df2d(ld_df(&Pw[ps[5] * LANES]));
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
                    f[k] = __ldg(&lt[(s0 + k) * LANES]);
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
                    f[k] = __ldg(&lt[(s0 + k) * LANES]);
                    a[k] = __ldg(&Aw[(s0 + k) * LANES]);
                    bb[k] = __ldg(&Bw[(s0 + k) * LANES]);
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
                    fwd_fast(s, Vw[s * LANES] + kt.x, kt.y, __ldg(&lt[s * LANES]));
                    pc += 9;
                    continue;
                }
                if (!GIV && ps[2] >= 0) {
                    passive(s, ps, R, D, K);
                    pc += 9;
                } else if (!chan_compartment_df<GIV, LANES>(v, E, cs, NR, pc, Vw[s * LANES], step, R, D)) {
                    if (v.status) atomicOr(v.status, ST_BAD_OP);
                    bad = true;
                    break;
                }
                fwd(s, R, D, __ldg(&lt[s * LANES]), __ldg(&Aw[s * LANES]), __ldg(&Bw[s * LANES]), K);
            }
        }
        if (split) {
            bar_named(1, 2 * LANES);   // the second warp's (R, D) of the rows above the static ones
            for (int s = nst; s < S; ++s)
                fwd(s, rdb[(2 * (s - nst)) * LANES], rdb[(2 * (s - nst) + 1) * LANES], __ldg(&lt[s * LANES]),
                    __ldg(&Aw[s * LANES]), __ldg(&Bw[s * LANES]), 0.0);
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
        double xn = 0.0;
        top = 0;
        // back substitution of row s: its solution from the parent's (the row
        // after, or the branch point on the stack)
        // (selects and predicated stack accesses instead of branches)
        // (TileType::slots: the stack entries come with the flags)
        auto bwd = [&](int s, int f, double2 rd, double c, double old) {
            const bool xl = f & FL_XLOAD;
            const int rs = ty.slots ? (f >> FL_SLOT_R) & 31 : (xl ? top - 1 : 0);
            const double sv = stk[rs * LANES];
            const double xp = xl ? sv : xn;
            if (!ty.slots) top -= (f & FL_XPOP) ? 1 : 0;
            double r = (f & FL_PARENT) ? fma(-c, xp, rd.x) : rd.x;
            r = r * rd.y;
            if (f & FL_XPUSH) stk[(ty.slots ? (f >> FL_SLOT_W) & 31 : top) * LANES] = r;
            if (!ty.slots) top += (f & FL_XPUSH) ? 1 : 0;
            xn = r;
            Vw[s * LANES] = ty.crank ? fma(2.0, r, -old) : r;
        };
        int s1 = S - 1;
        for (; s1 + 1 >= kCh; s1 -= kCh) {   // chunks: every row's loads, then the chain
            int f[kCh];
            double2 rd[kCh];
            double c[kCh], old[kCh];
#pragma unroll
            for (int k = 0; k < kCh; ++k) {
                const int s = s1 - k;
                f[k] = __ldg(&lt[s * LANES]);
                rd[k] = col[s * LANES];
                c[k] = __ldg(&Cbw[s * LANES]);
                old[k] = ty.crank ? Vw[s * LANES] : 0.0;
            }
#pragma unroll
            for (int k = 0; k < kCh; ++k) bwd(s1 - k, f[k], rd[k], c[k], old[k]);
        }
        for (; s1 >= 0; --s1)
            bwd(s1, __ldg(&lt[s1 * LANES]), col[s1 * LANES], __ldg(&Cbw[s1 * LANES]),
                ty.crank ? Vw[s1 * LANES] : 0.0);
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

inline cudaError_t stack_launch_mixed(const DevView &v, int tile0, int tile1, int cap, int nsteps, long long step,
                                      bool giv, bool split, cudaStream_t st)
{
    split = split && !giv;
    const size_t smem = ((size_t)cap + (split ? 2 * kSplitRows : 0)) * LANES * sizeof(double);
    auto fn = giv ? k_stack_mixed<true, false> : split ? k_stack_mixed<false, true> : k_stack_mixed<false, false>;
    if (smem > 48 * 1024) {
        const cudaError_t ce = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (ce != cudaSuccess) return ce;
    }
    fn<<<tile1 - tile0, split ? 2 * LANES : LANES, smem, st>>>(v, tile0, tile1, cap, nsteps, step);
    return cudaGetLastError();
}

// Wide tiles of the mixed form (see k_wide): the double-float lookups keep
// no bracket cache, so every compartment starts from a fresh cursor.
template <bool GIV>
__global__ void __launch_bounds__(32, 24)
k_wide_mixed(DevView v, int tile0, int tile1, int smax, int nsteps, long long step0)
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
    const int *sofs = v.prog + ty.wide_off;
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

    ChanEnvDF E;
    E.tab = v.tabdf + tg.tab_off;
    E.tg = tg;
    E.ncols = tg.ncols;
    E.xnmin = df_make(-tg.xmin_hi, -tg.xmin_lo);
    E.xinv = df_make(tg.invdx_hi, tg.invdx_lo);
    E.ynmin = df_make(-tg.ymin_hi, -tg.ymin_lo);
    E.yinv = df_make(tg.invdy_hi, tg.invdy_lo);
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
        for (int s = tid; s < S; s += nt) {
            ChanStateDF cs;
            chan_state_reset_df(cs);
            const int *pc = v.prog + sofs[s];
            double R = 0.0, D = 1.0;
            if (!chan_compartment_df<GIV, 1>(v, E, cs, NR, pc, V[s], step, R, D) && v.status)
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
        for (int l = 0; l < nf; ++l) {
            for (int i = fst[l] + tid; i < fst[l + 1]; i += nt) {
                const int s = frows[i];
                double d = Ds[s], r = Rs[s];
                for (int k = kst[s]; k < kst[s + 1]; ++k) {
                    const int c = kids[k];
                    const double temp = A[c] * Ds[c];   // Ds[c] holds the child's reciprocal
                    d = fma(-B[c], temp, d);
                    r = fma(-Rs[c], temp, r);
                }
                Ds[s] = rcp_newton(d);
                Rs[s] = r;
            }
            __syncthreads();
        }
        for (int l = 0; l < nb; ++l) {
            for (int i = bst[l] + tid; i < bst[l + 1]; i += nt) {
                const int s = brows[i];
                const int p = par[s];
                double r = Rs[s];
                if (p >= 0) r = fma(-Cb[s], Rs[p], r);
                r = r * Ds[s];
                Rs[s] = r;
                if (ty.crank) {
                    const double old = V[s];
                    V[s] = fma(2.0, r, -old);
                } else {
                    V[s] = r;
                }
            }
            __syncthreads();
        }
        if (tid == 0) finite_check(v, V[0], true);
    }
}

inline cudaError_t launch_mixed_impl(const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                                     long long step, bool giv, cudaStream_t st)
{
    const int ntiles = tile1 - tile0;
    const int blocks = (ntiles + warps - 1) / warps;
    const size_t smem = (size_t)warps * 2 * smax * LANES * sizeof(double);
    cudaError_t ce;
    if (giv) {
        if (smem > 48 * 1024) {
            ce = cudaFuncSetAttribute(k_steps_mixed<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (ce != cudaSuccess) return ce;
        }
        k_steps_mixed<true><<<blocks, warps * LANES, smem, st>>>(v, tile0, tile1, smax, nsteps, step);
    } else {
        if (smem > 48 * 1024) {
            ce = cudaFuncSetAttribute(k_steps_mixed<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (ce != cudaSuccess) return ce;
        }
        k_steps_mixed<false><<<blocks, warps * LANES, smem, st>>>(v, tile0, tile1, smax, nsteps, step);
    }
    return cudaGetLastError();
}

}  // namespace gbh
