// gbh_devfn.cuh -- device view of the engine's arrays and the helper
// functions shared by the interpreting kernels (gbh_kernels.cuh,
// gbh_kmixed.cuh) and the kernels generated per program at setup
// (gbh_jit.cu). Self-contained apart from gbh_internal.h and gbh_df.cuh so
// that the runtime compiler can build it without the CUDA headers.
#pragma once
#include "gbh_internal.h"
#include "gbh_df.cuh"

namespace gbh {

// A synchan whose synapses carry different weights: its events are kept as
// one bit per incoming synapse per future step (ring slot), the bits ranked
// in the order the reference sums them, and weight/dt of each rank.
struct SynW {
    int64_t mbase;   // word of slot 0 in DevView::wmask (slot q at mbase + q * nwords)
    int64_t wbase;   // weight/dt of rank 0 in DevView::wval
    int nwords;      // 32 ranks per word
    int pad;
};

struct DevView {
    const Tile *tiles;
    const TileType *types;
    const int *prog;
    const TableGeom *tgeom;
    const double *tab64;
    const float *tab32;
    const float4 *tabdf;     // per entry: table value and next-row difference, double-float
    const double *xyvals;
    double *P;        // parameter / state fields
    int *I;           // integer state (spike counters)
    double *V;        // vm
    double *C;        // conc
    double *F;        // flux (same rows as conc)
    const int *parent;   // topo rows: parent slot or -1
    const double *A, *B, *Cb;  // topo rows: forward A, forward B, backward C
    double *giv;      // givals rows
    // spikes and synaptic events
    unsigned *ring;           // event counts
    int ring_len;             // R
    const int64_t *syn_out_start;  // [neurons+1]
    const int64_t *syn_out_base;   // ring base of the target synchan (lane folded in)
    const int *syn_out_delay;      // effective delay in steps
    unsigned long long *spikes;    // per-neuron spike counter
    unsigned *spiked;              // per-neuron bit: spiked since the host last read it
    const double *stablist;        // synchan constants (shared by the batch)
    int *status;
    double dt;
    // Absolute step of launch-relative step 0, read on the device (kernels
    // replayed from a CUDA graph); null: the step0 argument is absolute.
    const long long *step_dev;
    // Grid barrier {arrivals, generation, abort} of a cooperative multi-step
    // launch (spikes cross tiles every step); null: no barrier.
    unsigned *gbar;
    // concentration rows beside C: coresult and codiag of each pool row
    // (diffusion systems), and per-lane scratch rows of the diffusion solves
    double *CR, *CD, *S;
    // wide tiles (one neuron per block): per-tile elimination schedules
    const int *wtop;
    // ravals rows of the solvers with symmetric compartments; itotal rows
    // of the storemode solvers
    double *RV, *IT;
    // Per-step host I/O inside a multi-step launch of the specialised kernels
    // (gbh_run_io): io_in[k * io_nin + i] is input i of step io_step0 + k and
    // io_out likewise. Per tile, tin_* list (offset in the tile's field block,
    // bit 30 set when the field is a packed double-float; input index) and
    // tout_* list (offset in its Vm block; output index). Null: none.
    const double *io_in;
    double *io_out;
    int io_nin, io_nout;
    long long io_step0;
    const int *tin_start, *tin_off, *tin_idx;
    const int *tout_start, *tout_off, *tout_idx;
    // stack elimination (TileType::stack): per-row flags (StackFlag), a
    // column of (right-hand side, diagonal or its reciprocal) per row, and
    // for the rows below nstatic their step-invariant (rhs term, coupling
    // factor), all at the tile's topo rows
    const int *ltop;
    double2 *col;
    double2 *kst;
    double *kri;   // FP64 form: the static rows' correctly rounded 1/D'
    // stack tiles' kept factors: the fields' generation (bumped by state
    // writes) and, per tile, the generation its kst / col were kept at
    const unsigned *sgen;
    unsigned *tgen;
    const int *kref;  // 1: an input writes a static row's Em/Rm, inject or dt/Cm; 2: also its diagonal term
    // synapses of weighted synchans (SynW): per synapse its bit's word for
    // slot 0 (-1 for a synchan of one weight) and bit | nwords << 5
    const int64_t *syn_out_mword;
    const int *syn_out_mbit;
    unsigned *wmask;
    const SynW *synw;
    const double *wval;
    // spike detection runs in a pass of its own before each step (k_spikes),
    // for networks with synapses that act in the step of the spike
    int spike_pre;
};

// A neuron whose Vm is no longer finite: a NaN or infinity anywhere in its
// tree reaches every row through the elimination within the step, so one
// row per neuron per step is checked (after back substitution). The mixed
// form's exact float<->double conversions run on the integer pipe and turn a
// NaN or infinity into a finite value near 2^128, so any |Vm| above 1e30 --
// no voltage in any unit system -- counts as lost as well.
__device__ __forceinline__ void finite_check(const DevView &v, double x, bool active)
{
    if (!(fabs(x) <= 1.0e30) && active && v.status) atomicOr(v.status, ST_NONFINITE);
}

// Named barrier `id` (1-15; 0 is __syncthreads') over `n` threads, a
// multiple of 32: warps that do different work in a step meet here from
// different places in the code.
__device__ __forceinline__ void bar_named(int id, int n)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Prefetch of the cache line holding *p into L1 (the loads of a later row).
__device__ __forceinline__ void prefetch_l1(const void *p)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// One synaptic event, counted in the target synchan's ring slot for the step
// it acts in; for a weighted synchan also its synapse's rank bit.
__device__ __forceinline__ void put_event(unsigned *ring, int ring_len, unsigned *wmask, int64_t base, int delay,
                                          int64_t mword, int mbit, long long step)
{
    const int slot = (int)((step + delay) % ring_len);
    atomicAdd(&ring[base + (int64_t)slot * LANES], 1u);
    if (mword >= 0) atomicOr(&wmask[mword + (int64_t)slot * (mbit >> 5)], 1u << (mbit & 31));
}

// h_dospike_event (hines_conn.c:44-58): an event on every synapse of the
// neuron, counted as a spike.
__device__ __forceinline__ void deliver_spike(const DevView &v, int64_t neuron, long long step)
{
    const int64_t e0 = v.syn_out_start[neuron], e1 = v.syn_out_start[neuron + 1];
    for (int64_t e = e0; e < e1; ++e)
        put_event(v.ring, v.ring_len, v.wmask, v.syn_out_base[e], v.syn_out_delay[e],
                  v.syn_out_mword ? v.syn_out_mword[e] : -1, v.syn_out_mbit ? v.syn_out_mbit[e] : 0, step);
    v.spikes[neuron] += 1ULL;
    if (v.spiked) atomicOr(&v.spiked[neuron >> 5], 1u << (neuron & 31));
}

// SPIKE_OP (hines_chip.c:266-276): the refractory counter counts down every
// step; above threshold with the counter spent, the neuron fires and the
// counter restarts. Returns the new counter.
__device__ __forceinline__ int spike_op(const DevView &v, double Vm, double thresh, int cnt, int refract,
                                        bool active, int64_t neuron, long long step)
{
    cnt -= 1;
    if (Vm > thresh && cnt <= 0 && active) {
        deliver_spike(v, neuron, step);
        cnt = refract;
    }
    return cnt;
}

// The events due now in one synchan's ring cell (h_dosynchan ->
// synchan HPROCESS, hines_conn.c:62-89, synchan.c:307-350): false if none;
// otherwise act = the sum of weight/dt over them, from zero, in the
// reference's order (its pending list puts a new event before the events
// due the same step, so the newest is summed first). w_dt >= 0: every
// synapse carries this weight/dt, one addition per event; w_dt < 0: the
// synchan has weights per synapse, described by synw[-w_dt - 1], its due
// bits summed in rank order. Clears what it consumed.
__device__ __forceinline__ bool syn_due(const DevView &v, unsigned *cell, double w_dt, long long step, double &act)
{
    const unsigned n = *cell;
    if (!n) return false;
    *cell = 0u;
    act = 0.0;
    if (w_dt >= 0.0) {
        for (unsigned q = 0; q < n; ++q) act += w_dt;
    } else {
        const SynW d = v.synw[(int64_t)(-w_dt) - 1];
        unsigned *m = v.wmask + d.mbase + (int64_t)(step % v.ring_len) * d.nwords;
        const double *w = v.wval + d.wbase;
        for (int k = 0; k < d.nwords; ++k) {
            unsigned b = m[k];
            m[k] = 0u;
            while (b) {
                const int j = __ffs(b) - 1;
                b &= b - 1;
                act += w[k * 32 + j];
            }
        }
    }
    return true;
}

// Elimination of one solver with symmetric compartments (SymOp program at
// sp, rows at stride STR): do_euler_hsolve / do_crank_hsolve
// (hines_solve.c:140-296) with the same operations in the same order,
// including the in-place updates of the ravals the program rewrites
// (COPY_ARRAY, FASTSIBARRAY_ELIM, SIBARRAY_ELIM). R and D hold each row's
// right-hand side and diagonal on entry, R the solution on exit; V is Vm.
// The decoder has checked every index against the solver's rows and ravals.
template <int STR>
__device__ __forceinline__ void sym_eliminate(const int *sp, double *R, double *D, double *RV, double *V, bool crank)
{
    int cur = 1;
    double rv = R[STR], dv = D[STR], temp = 0.0;
    for (;; sp += 3) {
        const int op = sp[0], a = sp[1], b = sp[2];
        if (op == SY_ELIM) {
            temp = RV[b * STR] / D[a * STR];
            dv -= RV[(b + 1) * STR] * temp;
            rv -= R[a * STR] * temp;
        } else if (op == SY_SET || op == SY_SKIP) {
            R[cur * STR] = rv;
            D[cur * STR] = dv;
            cur += op == SY_SET ? 1 : 2;
            rv = R[cur * STR];
            dv = D[cur * STR];
        } else if (op == SY_FASTSIB) {
            RV[a * STR] -= RV[b * STR] * temp;
        } else if (op == SY_COPY) {
            RV[a * STR] = RV[b * STR];
        } else if (op == SY_SIB) {
            RV[b * STR] -= RV[a * STR] * temp;
        } else {
            break;
        }
    }
    {
        const double x = rv / dv;
        V[cur * STR] = crank ? x + x - V[cur * STR] : x;
        R[cur * STR] = x;
    }
    cur -= 1;
    rv = R[cur * STR];
    for (sp += 3;; sp += 3) {
        const int op = sp[0], a = sp[1], b = sp[2];
        if (op == SY_ELIM) {
            rv -= RV[b * STR] * R[a * STR];
        } else if (op == SY_CALC) {
            const double x = rv / D[cur * STR];
            V[cur * STR] = crank ? x + x - V[cur * STR] : x;
            R[cur * STR] = x;
            cur -= 1;
            if (cur >= 0) rv = R[cur * STR];
        } else if (op == SY_SIB) {
            rv -= RV[a * STR] * R[b * STR];
        } else {
            break;
        }
    }
}

// Barrier over all blocks of a cooperative launch: the last block to arrive
// resets the count and advances the generation; the others wait for the
// generation to change, for at most ~2^22 polls (then they record
// ST_BARRIER, raise the abort word and leave, and so does every later
// barrier). Returns false once aborted.
__device__ __forceinline__ bool grid_sync(unsigned *bar, unsigned nblocks, int *status)
{
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = bar + 1;
        volatile unsigned *abort_w = bar + 2;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) == nblocks - 1) {
            bar[0] = 0u;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned polls = 0;
            while (*gen == g && !*abort_w) {
                if (++polls > (1u << 22)) {
                    atomicExch(bar + 2, 1u);
                    if (status) atomicOr(status, ST_BARRIER);
                    break;
                }
                if (polls > 4096) __nanosleep(64);   // spin first: steps are microseconds apart
            }
        }
        __threadfence();
        ok_s = *abort_w ? 0 : 1;
    }
    __syncthreads();
    return ok_s != 0;
}

// ---------------------------------------------------------------- helpers
struct VCursor {
    double lo, hi;
    int row, base;
    double frac;
};

__device__ __forceinline__ void locate(VCursor &c, double v, double vmin, double inv, int divs,
                                       const double *vals, int ncols, bool interp)
{
    if (interp) {
        double f = (v - vmin) * inv;
        if ((c.lo > v) || (v >= c.hi)) {
            if (f < 0.0)
                f = 0.0;
            else if (f > divs)
                f = divs;
            c.row = (int)f;
            f = f - (double)c.row;
            c.lo = vals[c.row];
            c.hi = vals[c.row + 1];
            c.base = c.row * ncols;
        } else {
            f = f - (double)c.row;
        }
        c.frac = f;
    } else {
        if ((c.lo > v) || (v >= c.hi)) {
            int k = (int)((v - vmin) * inv);
            if (k < 0)
                k = 0;
            else if (k > divs)
                k = divs;
            c.row = k;
            c.lo = vals[k];
            c.hi = vals[k + 1];
            c.base = k * ncols;
        }
        c.frac = 0.0;
    }
}

template <typename G>
__device__ __forceinline__ G gpow(G g, G x, int p)
{
    switch (p) {
    case 1: return g * x;
    case 2: return g * (x * x);
    case 3: return g * (x * x * x);
    case 4: x *= x; return g * (x * x);
    case 5: g *= x; x *= x; x *= x; return g * x;
    default: x *= x; g *= x; x *= x; return g * x;
    }
}

// Counter-based uniform deviate for SYN3_OP (statistical stand-in for G_RNG).
__device__ __forceinline__ double syn3_uniform(uint64_t key)
{
    key ^= key >> 33; key *= 0xff51afd7ed558ccdULL;
    key ^= key >> 33; key *= 0xc4ceb9fe1a85ec53ULL;
    key ^= key >> 33;
    return (double)(float)((double)(key >> 11) * (1.0 / 9007199254740992.0));
}

template <typename G> __device__ __forceinline__ const G *tab_ptr(const DevView &v, int64_t off);
template <> __device__ __forceinline__ const double *tab_ptr<double>(const DevView &v, int64_t off) { return v.tab64 + off; }
template <> __device__ __forceinline__ const float *tab_ptr<float>(const DevView &v, int64_t off) { return v.tab32 + off; }

struct DCursor {
    int row, base;
    df frac;
};

// table position of value v on an axis (min, inv) with divs rows, clamped
__device__ __forceinline__ void locate_df(DCursor &c, df v, df nmin, df inv, int divs, int ncols)
{
    df f = df_mul(df_add(v, nmin), inv);
    int row;
    if (f.hi <= 0.0f) {
        row = 0;
        f = df_make(0.f, 0.f);
    } else if (f.hi >= (float)divs) {
        row = divs;
        f = df_make(0.f, 0.f);
    } else {
        row = (int)floorf(f.hi);
        f = df_add_f(f, -(float)row);
        if (f.hi < 0.0f) {
            row -= 1;
            f = df_add_f(f, 1.0f);
        } else if (f.hi >= 1.0f) {
            row += 1;
            f = df_add_f(f, -1.0f);
        }
    }
    c.row = row;
    c.base = row * ncols;
    c.frac = f;
}

__device__ __forceinline__ df ld_df(const double *p)
{
    const float2 v = *reinterpret_cast<const float2 *>(p);
    return df_make(v.x, v.y);
}

// a row the kernel never writes during the launch (coefficients, gmax, Ek,
// tbyc, ...): read through the non-coherent path so the compiler may move the
// load ahead of the stores that precede it
__device__ __forceinline__ df ld_df_ro(const double *p)
{
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return df_make(v.x, v.y);
}

// a row the kernel itself may write between steps (the inject row, fused
// host I/O): read at L2, past L1, so a lane sees what another lane stored
__device__ __forceinline__ df ld_df_cg(const double *p)
{
    const float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
    return df_make(v.x, v.y);
}

// the same for a row read once per step (the unrolled form): first out of
// L1, which then keeps the table rows the gates gather from
__device__ __forceinline__ df ld_df_stream(const double *p)
{
    float2 v;
    asm("ld.global.nc.L1::evict_first.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
    return df_make(v.x, v.y);
}

__device__ __forceinline__ double ld_ro_stream(const double *p)
{
    double v;
    asm("ld.global.nc.L1::evict_first.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ int ld_ro_stream(const int *p)
{
    int v;
    asm("ld.global.nc.L1::evict_first.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// read-only view of a neuron-interleaved row array: r[i] loads through the
// non-coherent path
template <typename T>
struct RoRow {
    const T *p;
    __device__ __forceinline__ T operator[](int i) const { return __ldg(p + i); }
};

// read-only rows read once per step (the unrolled form): evict-first loads
template <typename T>
struct RoStream {
    const T *p;
    __device__ __forceinline__ T operator[](int i) const { return ld_ro_stream(p + i); }
};

__device__ __forceinline__ void st_df(double *p, df x)
{
    *reinterpret_cast<float2 *>(p) = make_float2(x.hi, x.lo);
}

// interpolated value of table entry e at fraction fr: value + fr*difference
__device__ __forceinline__ df interp_df(const float4 *tab, int e, df fr)
{
    const float4 t = __ldg(tab + e);
    return df_add(df_make(t.x, t.y), df_mul(df_make(t.z, t.w), fr));
}

__device__ __forceinline__ df val_df(const float4 *tab, int e)
{
    const float4 t = __ldg(tab + e);
    return df_make(t.x, t.y);
}

__device__ __forceinline__ df dpow(df g, df x, int p)
{
    switch (p) {
    case 1: return df_mul(g, x);
    case 2: return df_mul(g, df_mul(x, x));
    case 3: return df_mul(g, df_mul(df_mul(x, x), x));
    case 4: x = df_mul(x, x); return df_mul(g, df_mul(x, x));
    case 5: g = df_mul(g, x); x = df_mul(x, x); x = df_mul(x, x); return df_mul(g, x);
    default: x = df_mul(x, x); g = df_mul(g, x); x = df_mul(x, x); return df_mul(g, x);
    }
}



// ---- concentration pool phase (FP64 in every form) ------------------------
// Row views of one lane: conc C, flux F, coresult CR, codiag CD, fields P,
// vm V, scratch S (all neuron-interleaved, stride 32).
struct PoolLane {
    double *C, *F, *CR, *CD, *S;
    const double *P, *V;
    double dt;
    int crank;
};

__device__ __forceinline__ double hill_factor(int h, double X)
{
    return h == 2 ? X : h == 3 ? X * X : h == 4 ? X * X * X : 1.0;
}

// Shells without buffers, tridiagonal in the shell index (hines_conc.c:337-395).
// R: pool row of each shell, K: field row of each coupling term in the order
// consumed, fac/part: scratch rows.
template <int W>
__device__ __forceinline__ void diff_shells_dev(const PoolLane &L, int ms, const int *R, const int *K, int fac,
                                                int part)
{
#define GBH_C(j) L.C[R[j] * W]
#define GBH_CD(j) L.CD[R[j] * W]
#define GBH_CR(j) L.CR[R[j] * W]
#define GBH_K(q) L.P[K[q] * W]
    int q = 0, m;
    double up = GBH_K(q), dn, dd, f, x;
    q++;
    dd = up + GBH_CD(0);
    GBH_CD(0) = 1.0;
    L.S[part * W] = (GBH_C(0) + GBH_CR(0)) / dd;
    for (m = 1; m < ms - 1; m++) {
        f = -up / dd;
        L.S[(fac + m) * W] = f;
        dn = GBH_K(q);
        up = GBH_K(q + 1);
        q += 2;
        dd = GBH_CD(m) + dn * (1.0 + f) + up;
        GBH_CD(m) = 1.0;
        L.S[(part + m) * W] = (GBH_C(m) + GBH_CR(m) + dn * L.S[(part + m - 1) * W]) / dd;
    }
    f = -up / dd;
    L.S[(fac + m) * W] = f;
    dn = GBH_K(q);
    dd = GBH_CD(m) + dn * (1.0 + f);
    GBH_CD(m) = 1.0;
    x = (GBH_C(m) + GBH_CR(m) + dn * L.S[(part + m - 1) * W]) / dd;
    if (L.crank) {
        GBH_C(m) = x + x - GBH_C(m);
        for (m--; m >= 0; m--) {
            x = L.S[(part + m) * W] - L.S[(fac + m + 1) * W] * x;
            GBH_C(m) = x + x - GBH_C(m);
        }
    } else {
        GBH_C(m) = x;
        for (m--; m >= 0; m--) {
            x = L.S[(part + m) * W] - L.S[(fac + m + 1) * W] * x;
            GBH_C(m) = x;
        }
    }
}

// Shells with fixed and diffusible buffers (hines_conc.c:123-335): rows of a
// shell (nfix fixed buffers, diffusible buffers, the shell) eliminated as
// they are filled; BV: field rows of the buffer rates (3 per buffer).
// Scratch: fac[(shell*w + row)*w + column], part[shell*w + row].
template <int W>
__device__ __forceinline__ void diff_buffered_dev(const PoolLane &L, int ms, int w, int nfix, const int *R,
                                                  const int *K, const int *BV, int fac, int part)
{
#define GBH_F(i) L.S[(fac + (i)) * W]
#define GBH_PT(i) L.S[(part + (i)) * W]
#define GBH_B(i) L.P[BV[i] * W]
    const int w1 = w - 1, sq = w * w, last = ms - 1;
    int q = 0, m, n, nb, nc = 0, pr = 0, prev = -1, row = 0, srow = sq - w, sprev = srow - sq, cs = w1;
    double co = GBH_C(cs), dsh, rsh, dd, t, t2, h;
    for (m = 0; m < ms; m++) {
        dsh = GBH_CD(cs);
        GBH_CD(cs) = 1.0;
        rsh = GBH_CR(cs);
        for (n = 0, nb = 0; n < nfix; n++, nb += 3) {
            GBH_F(srow + n) = dd = GBH_B(nb) * co + GBH_B(nb + 1);
            dsh += t = GBH_B(nb) * GBH_C(nc);
            dd = 1.0 / (1.0 + dd);
            GBH_F(row) = t * dd;
            rsh += t2 = -GBH_B(nb + 1) * GBH_C(nc) + GBH_K(q);
            q++;
            GBH_PT(pr) = (GBH_C(nc) + t2) * dd;
            pr++;
            nc++;
            row += w;
        }
        for (; n < w1; n++, nb += 3) {
            GBH_F(srow + n) = dd = GBH_B(nb) * co + GBH_B(nb + 1);
            dsh += t = GBH_B(nb) * GBH_C(nc);
            rsh += t2 = -GBH_B(nb + 1) * GBH_C(nc) + GBH_B(nb + 2);
            if (m) {
                h = GBH_K(q) * GBH_F(row - sq);
                if (m < last) {
                    dd += 1.0 + GBH_K(q + 1) + GBH_K(q) * (1.0 + GBH_F(row - sq + 1)) - h * GBH_F(sprev + n);
                    GBH_F(row + 1) = -GBH_K(q + 1) / dd;
                    t2 += GBH_K(q) * GBH_C(nc - w) + (1.0 - GBH_K(q) - GBH_K(q + 1)) * GBH_C(nc) +
                          GBH_K(q + 1) * GBH_C(nc + w);
                } else {
                    dd += 1.0 + GBH_K(q) * (1.0 + GBH_F(row - sq + 1)) - h * GBH_F(sprev + n);
                    t2 += GBH_K(q) * GBH_C(nc - w) + (1.0 - GBH_K(q)) * GBH_C(nc);
                }
                GBH_PT(pr) = (t2 + GBH_K(q) * GBH_PT(pr - w) - h * GBH_PT(prev)) / dd;
                q += m < last ? 2 : 1;
            } else {
                dd += 1.0 + GBH_K(q);
                GBH_F(row + 1) = -GBH_K(q) / dd;
                GBH_PT(pr) = (t2 + (1.0 - GBH_K(q)) * GBH_C(nc) + GBH_K(q) * GBH_C(nc + w)) / dd;
                q++;
            }
            GBH_F(row) = t / dd;
            pr++;
            nc++;
            row += w;
        }
        if (m) {
            if (m < last) {
                dsh += GBH_K(q + 1) + GBH_K(q) * (1.0 + GBH_F(sprev + w1));
                rsh += GBH_K(q) * (GBH_C(nc - w) + GBH_PT(prev)) + (1.0 - GBH_K(q) - GBH_K(q + 1)) * co;
                cs += w;
                co = GBH_C(cs);
                rsh += GBH_K(q + 1) * co;
            } else {
                dsh += GBH_K(q) * (1.0 + GBH_F(sprev + w1));
                rsh += GBH_K(q) * (GBH_C(nc - w) + GBH_PT(prev)) + (1.0 - GBH_K(q)) * co;
            }
        } else {
            dsh += GBH_K(q);
            rsh += (1.0 - GBH_K(q)) * co;
            cs += w;
            co = GBH_C(cs);
            rsh += GBH_K(q) * co;
        }
        for (n = 0, nb = sprev; n < nfix; n++) {
            nb += w;
            prev++;
            dsh -= GBH_F(row + n) * GBH_F(nb);
            rsh -= GBH_F(row + n) * GBH_PT(prev);
        }
        for (; n < w1; n++) {
            nb += w;
            prev++;
            const double e = m ? GBH_F(row + n) + GBH_K(q) * GBH_F(sprev + n) : GBH_F(row + n);
            dsh -= e * GBH_F(nb);
            rsh -= e * GBH_PT(prev);
            if (m < last) GBH_F(row + n) *= -GBH_F(nb + 1);
        }
        if (m < last) {
            for (n = nfix; n < w1; n++) GBH_F(row + n) /= dsh;
            if (m) {
                GBH_F(row + w1) = -GBH_K(q + 1) / dsh;
                q += 2;
            } else {
                GBH_F(row + w1) = -GBH_K(q) / dsh;
                q++;
            }
            GBH_PT(pr) = rsh / dsh;
            prev = pr++;
            nc++;
            sprev = row;
            srow += sq;
            row += w;
        } else {
            co = GBH_C(nc) = rsh / dsh;
            nc--;
            q++;
        }
    }
    for (m = last; m >= 0; m--) {
        if (m < last) {
            row -= w;
            co = GBH_PT(--pr) - GBH_F(row + w1) * GBH_C(nc + w);
            for (n = nfix; n < w1; n++) co -= GBH_F(row + n) * GBH_C(nc + n + 1);
            GBH_C(nc) = co;
            nc--;
            for (n = w1; n > nfix; n--) {
                row -= w;
                GBH_C(nc) = GBH_PT(--pr) - GBH_F(row) * co - GBH_F(row + 1) * GBH_C(nc + w);
                nc--;
            }
        } else {
            for (n = w1; n > nfix; n--) {
                row -= w;
                GBH_C(nc) = GBH_PT(--pr) - GBH_F(row) * co;
                nc--;
            }
        }
        for (; n > 0; n--) {
            row -= w;
            GBH_C(nc) = GBH_PT(--pr) - GBH_F(row) * co;
            nc--;
        }
    }
#undef GBH_F
#undef GBH_PT
#undef GBH_B
#undef GBH_C
#undef GBH_CD
#undef GBH_CR
#undef GBH_K
}

// The pool program of one neuron (Ca_concen pools, concops groups, diffusion
// solves); W: row stride (32 lane-interleaved tiles, 1 wide tiles). Returns
// false on an unknown micro-op.
template <int W>
__device__ __forceinline__ bool pool_phase(const int *pp, const PoolLane &L)
{
    int ix = 0;
    double res = 0.0;
    while (pp[0] != 0) {
        switch (pp[0]) {
        case PO_CACONC: {
            double *cx = &L.C[pp[1] * W];
            const double base = L.P[pp[2] * W];
            const double itau = L.P[pp[3] * W];
            *cx = base + ((*cx - base) * (2.0 - itau) + (L.F[pp[1] * W] * L.P[pp[4] * W])) / itau;
            pp += 5;
            break;
        }
        case PO_GRP:
            ix = pp[1];
            res = 0.0;
            pp += 2;
            break;
        case PO_STORE:
            L.CR[ix * W] = res;
            pp += 1;
            break;
        case PO_FLUXCONC:
            res += L.P[pp[1] * W] + L.F[ix * W] * L.P[pp[2] * W];
            pp += 3;
            break;
        case PO_CTAU:
            res += L.P[pp[1] * W];
            L.CD[ix * W] += L.P[pp[2] * W];
            pp += 3;
            break;
        case PO_TAU: {
            const double itau = L.dt / (L.P[pp[2] * W] + L.P[pp[3] * W] *
                                        (exp((L.V[pp[1] * W] - L.P[pp[4] * W]) * L.P[pp[5] * W])));
            res += L.P[pp[6] * W] * itau;
            L.CD[ix * W] += itau;
            pp += 7;
            break;
        }
        case PO_MM:
            L.CD[ix * W] += L.P[pp[1] * W] / (L.C[ix * W] + L.P[pp[2] * W]);
            pp += 3;
            break;
        case PO_HILL: {
            const double X = L.C[ix * W];
            double c = hill_factor(pp[1], X);
            c = c / (c * X + L.P[pp[2] * W]);
            L.CD[ix * W] += L.P[pp[3] * W] * c;
            pp += 4;
            break;
        }
        case PO_PHILL: {
            const double X = L.C[pp[2] * W];
            double c = hill_factor(pp[1], X);
            c = c / (c * X + L.P[pp[3] * W]);
            L.CD[pp[2] * W] += L.P[pp[4] * W] * c;
            res += L.P[pp[5] * W] * c * X;
            pp += 6;
            break;
        }
        case PO_BUFFER: {
            double *bf = &L.C[pp[1] * W];
            const double X = L.P[pp[2] * W];
            const double c = ((1.0 - X) * *bf + L.P[pp[3] * W]) / (1.0 + X + L.P[pp[4] * W] * L.C[ix * W]);
            res += c - *bf;
            *bf = c;
            pp += 5;
            break;
        }
        case PO_POOL:
            L.C[ix * W] += res;
            pp += 1;
            break;
        case PO_DIFF: {
            const int ms = pp[1], w = pp[2], nfix = pp[3], sbase = pp[5], nq = pp[6], nb = pp[7];
            const int *R = pp + 8, *K = R + ms * w, *BV = K + nq;
            PoolLane L2 = L;
            L2.crank = pp[4];
            const int nfac = w > 1 ? ms * w * w : ms + 1;
            if (w > 1) diff_buffered_dev<W>(L2, ms, w, nfix, R, K, BV, sbase, sbase + nfac);
            else diff_shells_dev<W>(L2, ms, R, K, sbase, sbase + nfac);
            pp += 8 + ms * w + nq + nb;
            break;
        }
        default:
            return false;
        }
    }
    return true;
}
}  // namespace gbh
