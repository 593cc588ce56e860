// gbh_devfn.cuh -- device view of the engine's arrays and the helper
// functions shared by the interpreting kernels (gbh_kernels.cuh,
// gbh_kmixed.cuh) and the kernels generated per program at setup
// (gbh_jit.cu). Self-contained apart from gbh_internal.h and gbh_df.cuh so
// that the runtime compiler can build it without the CUDA headers.
#pragma once
#include "gbh_internal.h"
#include "gbh_df.cuh"

namespace gbh {

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
};

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

// read-only view of a neuron-interleaved row array: r[i] loads through the
// non-coherent path
template <typename T>
struct RoRow {
    const T *p;
    __device__ __forceinline__ T operator[](int i) const { return __ldg(p + i); }
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


}  // namespace gbh
