// gbh_engine.cu -- the GB300 hsolve engine: tile layout, device memory,
// launches, and the C ABI declared in include/gbhsolve.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "gbh_decode.h"
#include "gbh_kernels.cuh"
#include "gbh_df.cuh"
#include "gbh_jit.h"
#include "gbh_adjoint.h"
#include <thread>
#include "gbhsolve.h"

using namespace gbh;

namespace {

thread_local char g_last_error[320] = "no error";

void set_last(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            set_last("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return GBH_ERR_CUDA;                                                          \
        }                                                                                 \
    } while (0)

template <typename T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        n = count;
        if (count == 0) count = 1;
        if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
            set_last("cudaMalloc of %zu bytes failed", count * sizeof(T));
            return GBH_ERR_CUDA;
        }
        return GBH_OK;
    }
    int upload(const std::vector<T> &h)
    {
        if (alloc(h.size())) return GBH_ERR_CUDA;
        if (!h.empty()) CK(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
        return GBH_OK;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
    }
};

// A neuron's spike detector, for the pass before each step (k_spikes):
// element indices of its compartment's Vm, its threshold field and its
// counter rows, and its global neuron index.
struct SpikeSrc {
    int64_t vm, thresh, cnt, refr, neuron;
};

struct Launch {
    int tile0, tile1, smax, warps;
    int jit = -1;        // index of a specialised kernel, or -1 to interpret
    bool uniform = false; // every neuron of the type has the same tree
    bool wide = false;    // one neuron per block (wide tiles)
    bool stack = false;   // stack elimination (smax = shared doubles per lane)
    bool split = false;   // stack: some tile's rows above its static ones go to a second warp
};

// Element idx of a block of rows starting at row `base`: lane-interleaved
// tiles keep it at (base + idx) * 32 + lane, wide tiles (one neuron)
// contiguously at base * 32 + idx.
inline int64_t at(int64_t base, int64_t idx, int lane, bool wide)
{
    return wide ? base * LANES + idx : (base + idx) * LANES + lane;
}

// Rows a block of n elements takes in a tile.
inline int64_t rows_of(int64_t n, bool wide) { return wide ? (n + LANES - 1) / LANES : n; }

}  // namespace

struct gbh_engine {
    gbh_options opt{};
    int device = 0;
    int nsolvers = 0;
    double dt = 0.0;
    Decoded dec;
    std::vector<TileType> types;
    std::vector<Tile> tiles;
    std::vector<int> neuron_tile, neuron_lane;   // placement of every neuron
    std::vector<int64_t> chip_start, conc_start, ops_start, vm_start, giv_start, rav_start, itot_start;
    std::vector<double> chip_orig;              // reference chip[] for sync copies
    std::vector<int> ops_orig;
    int64_t ngiv_total = 0;
    // device buffers
    DBuf<Tile> d_tiles;
    DBuf<TileType> d_types;
    DBuf<int> d_prog;
    DBuf<TableGeom> d_tgeom;
    DBuf<double> d_tab64, d_xy;
    DBuf<float> d_tab32;
    DBuf<float4> d_tabdf;
    std::vector<std::vector<char>> type_df;     // mixed: field rows stored as packed double-float
    DBuf<double> d_P, d_V, d_C, d_F, d_A, d_B, d_Cb, d_giv, d_stab;
    DBuf<double> d_CR, d_CD, d_S;   // coresult / codiag rows, diffusion scratch
    DBuf<int> d_wtop;               // elimination schedules of wide tiles
    DBuf<double> d_RV;              // ravals rows of solvers with symmetric compartments
    DBuf<double> d_IT;              // itotal rows of storemode solvers
    DBuf<int> d_I, d_par;
    DBuf<int> d_ltop;              // stack elimination: per-row flags (topo rows)
    DBuf<double2> d_col;           // stack elimination: (rhs, diagonal) per row
    DBuf<double2> d_kst;           // stack elimination: static rows' (rhs term, coupling factor)
    DBuf<double> d_kri;            // stack elimination, FP64 form: static rows' 1/D'
    DBuf<unsigned> d_sgen, d_tgen; // stack elimination: the fields' generation; each tile's kept one
    unsigned sgen_host = 1;
    std::vector<std::vector<char>> stack_dfield;   // per type: field rows that are a static row's diagonal term
    std::vector<std::vector<char>> stack_kfield;   // per type: field rows of a static row's rhs term
    bool stack_input_d = false;    // an input writes such a field: every launch redoes the kept factors
    DBuf<int> d_kref;              // an input writes a static row's rhs fields: launches refresh them
    DBuf<unsigned> d_ring;
    DBuf<int64_t> d_out_start, d_out_base;
    DBuf<int> d_out_delay;
    // synchans whose synapses carry different weights (SynW)
    DBuf<int64_t> d_out_mword, d_rmword;
    DBuf<int> d_out_mbit, d_rmbit;
    DBuf<SynW> d_synw;
    DBuf<double> d_wval;
    DBuf<unsigned> d_wmask;
    // spike detection in a pass of its own (synapses acting in the spike's step)
    bool spike_pre = false;
    int nspike_src = 0;
    DBuf<SpikeSrc> d_spike_src;
    DBuf<unsigned long long> d_spikes;
    // networks: cooperative multi-step launches (grid barrier every step)
    DBuf<unsigned> d_gbar;
    bool net_coop = false;
    int net_spl = 1;
    // partitioned networks: spikes recorded per neuron, remote-source synapses
    DBuf<unsigned> d_spiked;
    int nremote = 0;
    DBuf<int64_t> d_rstart, d_rbase;
    DBuf<int> d_rdelay;
    DBuf<unsigned char> d_rbits;
    DBuf<int> d_status;
    int ring_len = 2;
    int64_t rows_fld = 0, rows_int = 0, rows_pool = 0, rows_giv = 0, rows_vm = 0, rows_topo = 0,
            rows_syn = 0, rows_scr = 0, rows_rav = 0, rows_itot = 0;
    std::vector<Launch> launches;
    int steps_per_launch = 1;
    bool has_network = false;
    bool givals_enabled = false;
    bool givals_valid = false;
    long long step = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    gbh_stats stats{};
    std::vector<JitKernel> jits;                 // active kernel of each specialised type
    std::vector<std::vector<JitKernel>> jit_var;  // compiled variants per specialised type
    std::vector<int> jit_minb;                    // residency target of each variant
    std::vector<char> jit_compact;                // variant is the compact (looped) form
    std::vector<char> jit_smemrows;               // variant keeps the unrolled form's rows in shared memory
    std::vector<int> jit_warps;                   // warps per block of each variant
    int jit_choice = 0;
    int jit_compiled = 0;
    std::string jit_log;
    // CUDA graphs of whole runs (opt.use_graph): one per (steps, steps per
    // launch, kernel variant); the step number lives on the device
    struct Graph {
        int nsteps, spl, variant;
        cudaGraphExec_t exec;
        int64_t kernels;
    };
    std::vector<Graph> graphs;
    cudaStream_t cap_stream = nullptr;
    // side streams: launch groups (tile types) run concurrently
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> ev_join;
    cudaEvent_t ev_fork = nullptr;
    DBuf<long long> d_step;
    bool dstep_valid = false;
    // pipelined per-step I/O (gbh_step_io): host->device and device->host
    // copies each on their own stream (one FIFO would put a step's input copy
    // behind the previous step's output copy), double-buffered staging
    cudaStream_t io_stream = nullptr, io_out_stream = nullptr;
    DBuf<double> d_io_in[2], d_io_out[2];
    cudaEvent_t io_in_copied[2] = {nullptr, nullptr}, io_gathered[2] = {nullptr, nullptr},
                io_out_copied[2] = {nullptr, nullptr};
    long long io_calls = 0;
    int io_nin = -1, io_nout = -1;
    // block-streamed I/O (gbh_run_io): staging for `blk_cap` steps of inputs
    // and outputs, double-buffered
    DBuf<double> d_blk_in[2], d_blk_out[2];
    cudaEvent_t blk_in_copied[2] = {nullptr, nullptr}, blk_done[2] = {nullptr, nullptr},
                blk_out_copied[2] = {nullptr, nullptr};
    int blk_cap = 0, blk_nin = -1, blk_nout = -1;
    // the previous call's output gather, issued together with the next
    // call's input scatter (one kernel between two steps)
    double *io_pend_host = nullptr;
    int io_pend_buf = 0;
    cudaStream_t io_pend_stream = nullptr;
    // per-step I/O (h_in_msgs / h_out_msgs)
    int n_in = 0, n_out = 0, n_tgt = 0;   // input values, distinct input targets, outputs
    DBuf<double> d_in_vals, d_out_vals, d_in_sa, d_in_sb;
    DBuf<int64_t> d_in_start, d_in_addr, d_out_addr;
    DBuf<int> d_in_item;
    // the same inputs / outputs as per-tile lists for the specialised kernels,
    // which apply them inside multi-step launches (gbh_run_io); fuse_in: every
    // input sets a compartment's inject (the row those kernels read coherently)
    DBuf<int> d_tin_start, d_tin_off, d_tin_idx, d_tout_start, d_tout_off, d_tout_idx;
    bool fuse_in = false;
};

// The spike-detection pass before a step (k_spikes), on stream st.
int launch_spikes(gbh_engine *e, const gbh::DevView &v, long long step, cudaStream_t st);

namespace {

int fail_err(gbh_error *err, int code, const char *fmt, ...)
{
    char buf[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (err) {
        err->code = code;
        err->solver = err->row = -1;
        err->opcode = 0;
        err->position = -1;
        snprintf(err->message, sizeof(err->message), "%s", buf);
    }
    set_last("%s", buf);
    return code;
}

// Operand counts of the engine micro-ops (see gbh_internal.h).
int micro_operands(int code)
{
    switch (code) {
    case M_BEGIN: return 4;
    case M_NEWVOLT: case M_NEWCONC1: case M_FLUX: case M_DO_TABGHK: return 0;
    case M_CONCVAL: case M_DOMAIN: case M_NEWCONC2: case M_SCALE_FLUX: case M_SAME_GHK:
    case M_CHAN_G: case M_ADDCURR: return 1;
    case M_NERNST: case M_CHAN: case M_STORE: return 2;
    case M_SPIKE: case M_GHK: case M_END: case M_ITLEAK: return 3;
    case M_ELMMPUMP: case M_GATE: case M_MGBLOCK: return 4;
    case M_SYN: return 6;
    default: return -1;
    }
}

// Which operands of a micro-op are field rows (bit i: operand i).
int field_operands(int code)
{
    switch (code) {
    case M_BEGIN: return 0x7;
    case M_DOMAIN: case M_SCALE_FLUX: case M_SAME_GHK: case M_CHAN_G: return 0x1;
    case M_SPIKE: return 0x1;
    case M_ELMMPUMP: return 0x7;
    case M_GHK: return 0x7;
    case M_NERNST: case M_CHAN: case M_END: case M_ITLEAK: return 0x3;
    case M_GATE: return 0x8;
    case M_SYN: return 0x39;
    case M_MGBLOCK: return 0x7;
    default: return 0;
    }
}

// Per slot of a type's program, 6 ints for the stack kernels: the first and
// last field row it reads (rows are allocated in program order, so a slot's
// fields are mostly one contiguous range; prefetched a few rows ahead), and
// for a passive compartment -- a program of M_BEGIN and M_END alone -- the
// rows of Em/Rm, inject, dt/Cm and the diagonal term (else -1): such rows
// skip the interpreter.
std::vector<int> slot_field_ranges(const std::vector<int> &prog, const TileType &tt)
{
    std::vector<int> out;
    size_t pc = tt.prog_off;
    for (int s = 0; s < tt.nslots; ++s) {
        int lo = INT32_MAX, hi = -1;
        const size_t pc0 = pc;
        const bool passive = prog[pc0] == M_BEGIN && prog[pc0 + 5] == M_END;
        for (;;) {
            const int code = prog[pc];
            const int n = micro_operands(code);
            if (n < 0) break;
            const int fm = field_operands(code);
            for (int i = 0; i < n; ++i)
                if ((fm >> i) & 1) {
                    const int f = prog[pc + 1 + i];
                    if (f >= 0) {
                        lo = std::min(lo, f);
                        hi = std::max(hi, f);
                    }
                }
            pc += 1 + n;
            if (code == M_END) break;
        }
        if (hi < 0) lo = hi = 0;
        out.push_back(lo);
        out.push_back(std::min(hi, lo + 31));
        if (passive) {
            out.push_back(prog[pc0 + 1]);   // Em/Rm
            out.push_back(prog[pc0 + 2]);   // inject
            out.push_back(prog[pc0 + 6]);   // dt/Cm
            out.push_back(prog[pc0 + 7]);   // diagonal term
        } else {
            out.insert(out.end(), {-1, -1, -1, -1});
        }
    }
    return out;
}

// Slot and rows of the spike detector in a type's program (M_SPIKE operands:
// threshold field, counter and refractory int rows).
bool spike_rows(const std::vector<int> &prog, const TileType &tt, int &slot, int &fth, int &icnt, int &iref)
{
    size_t pc = tt.prog_off;
    for (int s = 0; s < tt.nslots; ++s) {
        for (;;) {
            const int code = prog[pc];
            const int n = micro_operands(code);
            if (n < 0) return false;
            if (code == M_SPIKE) {
                slot = s;
                fth = prog[pc + 1];
                icnt = prog[pc + 2];
                iref = prog[pc + 3];
                return true;
            }
            pc += 1 + n;
            if (code == M_END) break;
        }
    }
    return false;
}

// Fields the mixed-precision kernel reads as packed double-float pairs.
std::vector<char> df_fields_of(const TileType &tt, const std::vector<int> &prog)
{
    std::vector<char> m(tt.nfields, 0);
    size_t pc = tt.prog_off;
    for (int s = 0; s < tt.nslots; ++s) {
        for (;;) {
            const int code = prog[pc];
            const int n = micro_operands(code);
            if (n < 0) return m;
            const int *o = &prog[pc + 1];
            if (code == M_BEGIN) { m[o[0]] = 1; m[o[1]] = 1; }
            else if (code == M_CHAN) { m[o[0]] = 1; m[o[1]] = 1; }
            else if (code == M_CHAN_G) { m[o[0]] = 1; }
            else if (code == M_GATE && o[2] != 0) { m[o[3]] = 1; }
            else if (code == M_END) { m[o[0]] = 1; m[o[1]] = 1; }
            pc += 1 + n;
            if (code == M_END) break;
        }
    }
    return m;
}

double pack_df(double x)
{
    const float hi = (float)x;
    const float lo = (float)(x - (double)hi);
    float2 f = make_float2(hi, lo);
    double d;
    memcpy(&d, &f, sizeof(d));
    return d;
}

double unpack_df(double d)
{
    float2 f;
    memcpy(&f, &d, sizeof(d));
    return (double)f.x + (double)f.y;
}

// Shared-memory budget per block for the elimination columns.
constexpr int kSmemPerBlock = 96 * 1024;
// Lane-mapped types of at least this many compartments that are not
// specialised run the stack elimination (k_stack*) rather than the
// interpreter's shared-memory columns (2 x compartments x 32 doubles a warp).
// From 8: the random trees of 8-31 compartments beside the larger ones ran
// 6 % faster that way (their passive rows take the static-row fast path).
constexpr int kStackMin = 8;
// Shared memory a stack-elimination warp may take (doubles per lane).
constexpr int kStackCapMax = 200 * 1024 / (LANES * (int)sizeof(double)) - 2 * kSplitRows;

// Composite tables on the device: FP64 copy (plus one padding row), axis
// value pools and their geometry.
void build_tables(const gbh_batch_desc *d, std::vector<TableGeom> &tg, std::vector<double> &tab64,
                  std::vector<double> &xy)
{
    tg.assign(d->ntables, TableGeom{});
    for (int k = 0; k < d->ntables; ++k) {
        const gbh_tables &T = d->tables[k];
        TableGeom g{};
        g.ncols = T.ncols;
        g.xdivs = T.xdivs;
        g.ydivs = T.ydivs;
        g.xmin = T.xmin;
        g.invdx = T.invdx;
        g.ymin = T.ymin;
        g.invdy = T.invdy;
        g.tab_off = (int64_t)tab64.size();
        const int64_t rows = T.ncols ? (int64_t)T.xdivs + 1 : 0;
        for (int64_t r = 0; r < rows; ++r)
            for (int cc = 0; cc < T.ncols; ++cc) tab64.push_back(T.tablist[r * T.ncols + cc]);
        // one padding row: the clamped top row reads row xdivs+1
        for (int cc = 0; cc < T.ncols; ++cc) tab64.push_back(rows ? T.tablist[(rows - 1) * T.ncols + cc] : 0.0);
        g.xv_off = (int64_t)xy.size();
        for (int64_t r = 0; r < rows; ++r) xy.push_back(T.xvals[r]);
        xy.push_back(rows ? T.xvals[rows - 1] : 0.0);   // empty top bracket: always relocate
        xy.push_back(0.0);
        g.yv_off = -1;
        if (T.ydivs > 0 && T.yvals) {
            g.yv_off = (int64_t)xy.size();
            for (int r = 0; r <= T.ydivs; ++r) xy.push_back(T.yvals[r]);
            xy.push_back(T.yvals[T.ydivs]);
            xy.push_back(0.0);
        }
        tg[k] = g;
    }
    for (TableGeom &g : tg) {
        auto split = [](double x, float &h, float &l) { h = (float)x; l = (float)(x - (double)h); };
        split(g.xmin, g.xmin_hi, g.xmin_lo);
        split(g.invdx, g.invdx_hi, g.invdx_lo);
        split(g.ymin, g.ymin_hi, g.ymin_lo);
        split(g.invdy, g.invdy_hi, g.invdy_lo);
    }
}

// Can a type run wide (its compartments on separate threads)? Each
// compartment must start from nothing but the table cursors the chain of
// NEWVOLT / NEWCONC1 lookups leaves (resolved per step in the kernel): no
// DOMAIN / NEWCONC2 / 2-D tables / TABGHK / SAME_GHK, a CONC_VAL before
// anything that uses the selected conc, a current before FLUX, a lookup
// before a gate that reads its cursor, at most one lookup of each kind per
// compartment. On success meta = [program offset of each slot | previous
// NEWVOLT slot (-1 none, -2 the slot has none) | same for NEWCONC1 | conc
// row NEWCONC1 reads].
bool wide_plan(const std::vector<int> &prog, const TileType &tt, std::vector<int> &meta)
{
    const int S = tt.nslots;
    std::vector<int> sofs(S), vprev(S, -2), cprev(S, -2), cpool(S, 0);
    size_t pc = tt.prog_off;
    int lastv = -1, lastc = -1;
    for (int s = 0; s < S; ++s) {
        sofs[s] = (int)pc;
        bool sel = false, ik = false;
        int nv = 0, nc = 0, selrow = 0;
        for (;;) {
            const int code = prog[pc];
            const int n = micro_operands(code);
            if (n < 0) return false;
            const int *o = &prog[pc + 1];
            switch (code) {
            case M_DOMAIN: case M_NEWCONC2: case M_SAME_GHK: case M_DO_TABGHK: case M_STORE: case M_ITLEAK:
                return false;
            case M_CONCVAL: sel = true; selrow = o[0]; break;
            case M_NEWVOLT: if (++nv > 1) return false; break;
            case M_NEWCONC1:
                if (!sel || ++nc > 1) return false;
                cpool[s] = selrow;
                break;
            case M_ELMMPUMP: if (!sel) return false; ik = true; break;
            case M_GHK: case M_NERNST: if (!sel) return false; break;
            case M_FLUX: case M_SCALE_FLUX: if (!sel || !ik) return false; break;
            case M_GATE:
                if (o[0] == GK_2V || o[0] == GK_2C) return false;
                if ((o[0] == GK_1V && !nv) || (o[0] == GK_1C && !nc)) return false;
                break;
            case M_ADDCURR: ik = true; break;
            default: break;
            }
            pc += 1 + n;
            if (code == M_END) break;
        }
        if (nv) { vprev[s] = lastv; lastv = s; }
        if (nc) { cprev[s] = lastc; lastc = s; }
    }
    meta = sofs;
    meta.insert(meta.end(), vprev.begin(), vprev.end());
    meta.insert(meta.end(), cprev.begin(), cprev.end());
    meta.insert(meta.end(), cpool.begin(), cpool.end());
    return true;
}

// Stack elimination plan of one neuron (see k_stack): per-row StackFlag words
// and the shared memory the two stacks need, in doubles per lane. Returns
// false unless the rows are a post-order of the tree -- each row's last
// child the row before it, its other children the top entries of the
// forward stack, and on the way back the parent's solution on the top of the
// backward stack -- which the Hines numbering of do_hnum
// (hines_init.c:317-345) always gives; the neuron then runs another kernel.
bool stack_plan(const std::vector<int> &parent, std::vector<int> &flags, int &cap)
{
    const int S = (int)parent.size();
    std::vector<int> nk(S, 0), first(S, -1);
    for (int s = 0; s < S; ++s) {
        const int p = parent[s];
        if (p < 0) continue;
        if (p <= s || p >= S) return false;
        if (nk[p]++ == 0) first[p] = s;
    }
    flags.assign(S, 0);
    std::vector<int> st;
    size_t fmax = 0, bmax = 0;
    for (int s = 0; s < S; ++s) {
        int f = 0;
        if (nk[s] > 0) {
            const int np = nk[s] - 1;
            if (parent[s - 1] != s || np > FL_NPOP || (int)st.size() < np) return false;
            for (int j = 0; j < np; ++j)
                if (parent[st[st.size() - np + j]] != s) return false;
            st.resize(st.size() - np);
            f |= np | FL_CARRY_IN;
        }
        if (parent[s] >= 0) {
            f |= FL_PARENT;
            if (parent[s] == s + 1) {
                f |= FL_CARRY_OUT;
            } else {
                f |= FL_PUSH;
                st.push_back(s);
                fmax = std::max(fmax, st.size());
            }
        }
        flags[s] = f;
    }
    if (!st.empty()) return false;
    for (int s = S - 1; s >= 0; --s) {
        const int p = parent[s];
        if (p >= 0 && p != s + 1) {
            if (st.empty() || st.back() != p) return false;
            flags[s] |= FL_XLOAD;
            if (first[p] == s) {
                flags[s] |= FL_XPOP;
                st.pop_back();
            }
        }
        if (nk[s] >= 2) {
            flags[s] |= FL_XPUSH;
            st.push_back(s);
            bmax = std::max(bmax, st.size());
        }
    }
    if (!st.empty()) return false;
    cap = (int)std::max<size_t>(std::max(2 * fmax, bmax), 1);
    return true;
}

// The stack entry of every row (TileType::slots), from its flags: forward,
// the depth after its pops; backward, the entry it reads its parent's
// solution from and the one it writes its own to. False when one is 32 or
// more. `fdepth`: the largest forward entry index used.
bool stack_slots(const std::vector<int> &flags, std::vector<int> &packed, int &fdepth)
{
    const int S = (int)flags.size();
    packed.assign(S, 0);
    fdepth = 0;
    int top = 0;
    for (int s = 0; s < S; ++s) {
        const int f = flags[s];
        top -= f & FL_NPOP;
        if (top < 0 || top > 31) return false;
        packed[s] |= top << FL_SLOT_F;
        fdepth = std::max(fdepth, top);
        if (f & FL_PUSH) ++top;
    }
    top = 0;
    for (int s = S - 1; s >= 0; --s) {
        const int f = flags[s];
        const int rb = (f & FL_XLOAD) ? top - 1 : 0;
        if (f & FL_XPOP) --top;
        if (rb < 0 || rb > 31 || top < 0 || top > 31) return false;
        packed[s] |= rb << FL_SLOT_R | top << FL_SLOT_W;
        if (f & FL_XPUSH) ++top;
    }
    return true;
}

// Elimination schedule of one wide neuron (see k_wide): forward levels by
// height (leaves 0), children of each row in ascending order, backward
// levels by depth (root 0).
void wide_schedule(const std::vector<int> &parent, std::vector<int> &out)
{
    const int S = (int)parent.size();
    std::vector<int> h(S, 0), dep(S, 0);
    for (int s = 0; s < S; ++s)   // children have lower rows than their parents
        if (parent[s] >= 0) h[parent[s]] = std::max(h[parent[s]], h[s] + 1);
    for (int s = S - 1; s >= 0; --s)
        if (parent[s] >= 0) dep[s] = dep[parent[s]] + 1;
    auto levels = [&](const std::vector<int> &lv, std::vector<int> &start, std::vector<int> &rows) {
        const int nl = S ? *std::max_element(lv.begin(), lv.end()) + 1 : 0;
        start.assign(nl + 1, 0);
        for (int s = 0; s < S; ++s) start[lv[s] + 1]++;
        for (int l = 0; l < nl; ++l) start[l + 1] += start[l];
        rows.assign(S, 0);
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int s = 0; s < S; ++s) rows[fill[lv[s]]++] = s;
        return nl;
    };
    std::vector<int> fs, fr, bs, br;
    const int nf = levels(h, fs, fr), nb = levels(dep, bs, br);
    std::vector<int> kst(S + 1, 0), kids;
    for (int s = 0; s < S; ++s)
        if (parent[s] >= 0) kst[parent[s] + 1]++;
    for (int s = 0; s < S; ++s) kst[s + 1] += kst[s];
    kids.assign(std::max(S - 1, 0), 0);
    std::vector<int> fill(kst.begin(), kst.end() - 1);
    for (int s = 0; s < S; ++s)   // ascending: the order the sequential sweep applies them
        if (parent[s] >= 0) kids[fill[parent[s]]++] = s;
    out.clear();
    out.push_back(nf);
    out.insert(out.end(), fs.begin(), fs.end());
    out.insert(out.end(), fr.begin(), fr.end());
    out.insert(out.end(), kst.begin(), kst.end());
    out.insert(out.end(), kids.begin(), kids.end());
    out.push_back(nb);
    out.insert(out.end(), bs.begin(), bs.end());
    out.insert(out.end(), br.begin(), br.end());
}

int build_layout(gbh_engine *e, const gbh_batch_desc *d, const gbh_synapses *syn, const gbh_remote_synapses *remote,
                 gbh_error *err)
{
    Decoded &dec = e->dec;
    const int nneu = (int)dec.neurons.size();
    // ---- group neurons by program signature ----
    std::map<std::string, int> type_of_key;
    std::vector<std::vector<int>> members;
    std::vector<int> prog_pool;
    for (int i = 0; i < nneu; ++i) {
        auto it = type_of_key.find(dec.neurons[i].key);
        if (it == type_of_key.end()) {
            const Neuron &N = dec.neurons[i];
            TileType tt{};
            tt.nslots = N.nrows;
            tt.nfields = (int)N.fsrc.size();
            tt.nints = (int)N.iops.size();
            tt.npools = (int)N.pool_conc.size();
            tt.ngiv = (int)N.giv_ref.size();
            tt.prog_off = (int)prog_pool.size();
            prog_pool.insert(prog_pool.end(), N.prog.begin(), N.prog.end());
            tt.pool_off = (int)prog_pool.size();
            prog_pool.insert(prog_pool.end(), N.pool_prog.begin(), N.pool_prog.end());
            tt.table_set = N.table_set;
            tt.crank = N.crank;
            tt.chanmode5 = N.c5;
            tt.interp = N.interp;
            tt.has_spike = N.spike_op >= 0;
            tt.nsyn = (int)N.syn_op.size();
            tt.has_cd = N.has_cd;
            tt.nscratch = N.nscratch;
            if (!N.sym.empty()) {
                tt.sym = 1;
                tt.sym_off = (int)prog_pool.size();
                prog_pool.insert(prog_pool.end(), N.sym.begin(), N.sym.end());
                tt.nrav = (int)N.rav.size();
            }
            tt.nitot = N.nitot;
            type_of_key[N.key] = (int)e->types.size();
            e->types.push_back(tt);
            members.emplace_back();
            it = type_of_key.find(N.key);
        }
        members[it->second].push_back(i);
    }
    // ---- wide types: one neuron per tile, its compartments on a block's threads ----
    if (e->opt.wide_min >= 0) {
        // Default 32 compartments. Measured (compartment-steps/s, mixed / FP64):
        // 50,000 random trees of 8-256 compartments, threshold 32: 8.5e9 / 2.9e9;
        // 16 (for types of fewer than 1,024 neurons): 8.1e9 / 2.6e9; all
        // lane-mapped (10,000 trees): 1.2e9 / 0.9e9. 1,000 16-compartment
        // cables ran 20 % slower one per warp than 32 per warp.
        for (size_t ti = 0; ti < e->types.size(); ++ti) {
            TileType &tt = e->types[ti];
            const bool by_size = tt.nslots >= (e->opt.wide_min > 0 ? e->opt.wide_min : 32) && !tt.sym && !tt.nitot;
            std::vector<int> meta;
            if (by_size && wide_plan(prog_pool, tt, meta)) {
                tt.wide = 1;
                tt.wide_off = (int)prog_pool.size();
                prog_pool.insert(prog_pool.end(), meta.begin(), meta.end());
            }
        }
    }
    // ---- stack elimination for the remaining large lane-mapped types ----
    for (size_t ti = 0; ti < e->types.size(); ++ti) {
        TileType &tt = e->types[ti];
        if (tt.wide || tt.sym || tt.nslots < kStackMin) continue;
        int cap = 2;   // at least one stack entry: the sweeps read an entry whether or not they use it
        bool ok = true, np1 = true, slots = true;
        std::vector<int> fl, sl;
        for (int i : members[ti]) {
            int c = 0, fdepth = 0;
            if (!stack_plan(dec.neurons[i].parent, fl, c)) {
                ok = false;
                break;
            }
            cap = std::max(cap, c);
            for (int f : fl) np1 = np1 && (f & FL_NPOP) <= 1;
            // the forward sweep reads its row's entry whether or not it pops
            if (slots && stack_slots(fl, sl, fdepth)) cap = std::max(cap, 2 * fdepth + 2);
            else slots = false;
        }
        if (ok && cap <= kStackCapMax) {
            tt.stack = 1;
            tt.scap = cap;
            tt.np1 = np1;
            tt.slots = np1 && slots;
            const std::vector<int> pf = slot_field_ranges(prog_pool, tt);
            tt.nstatic = 0;
            while (tt.nstatic < tt.nslots && pf[6 * tt.nstatic + 2] >= 0) ++tt.nstatic;
            e->stack_dfield.resize(e->types.size());
            e->stack_kfield.resize(e->types.size());
            e->stack_dfield[ti].assign(tt.nfields, 0);
            e->stack_kfield[ti].assign(tt.nfields, 0);
            for (int q = 0; q < tt.nstatic; ++q) {
                if (pf[6 * q + 5] >= 0 && pf[6 * q + 5] < tt.nfields) e->stack_dfield[ti][pf[6 * q + 5]] = 1;
                for (int c = 2; c <= 4; ++c)   // Em/Rm, inject, dt/Cm
                    if (pf[6 * q + c] >= 0 && pf[6 * q + c] < tt.nfields) e->stack_kfield[ti][pf[6 * q + c]] = 1;
            }
            tt.pf_off = (int)prog_pool.size();
            prog_pool.insert(prog_pool.end(), pf.begin(), pf.end());
        }
    }
    // ---- event ring length from the synapse delays ----
    const bool local_syn = syn && syn->nsynapses > 0;
    const int64_t nrsyn = (remote && remote->nsources > 0) ? remote->src_start[remote->nsources] : 0;
    e->has_network = local_syn || nrsyn > 0 || (remote && remote->nsources > 0);
    int maxd = 1;
    if (local_syn) {
        for (int64_t s = 0; s < syn->nsynapses; ++s) {
            // (int)(delay/dt + 0.9) steps (synchan.c:199-200): zero for a delay under 0.1 dt
            if (syn->delay_steps[s] < 0)
                return fail_err(err, GBH_ERR_ARG, "synapse %lld has a negative delay", (long long)s);
            maxd = std::max(maxd, syn->delay_steps[s] + 1);
        }
    }
    for (int64_t k = 0; k < nrsyn; ++k) {
        if (remote->delay_steps[k] < 1)
            return fail_err(err, GBH_ERR_UNSUPPORTED, "remote synapse %lld has a delay below one step",
                            (long long)k);
        maxd = std::max(maxd, remote->delay_steps[k]);
    }
    e->ring_len = maxd + 1;
    // ---- tiles: types ordered by slot count (descending) ----
    std::vector<int> torder(e->types.size());
    for (size_t i = 0; i < torder.size(); ++i) torder[i] = (int)i;
    std::stable_sort(torder.begin(), torder.end(),
                     [&](int a, int b) { return e->types[a].nslots > e->types[b].nslots; });
    e->neuron_tile.assign(nneu, -1);
    e->neuron_lane.assign(nneu, -1);
    int64_t gneuron = 0;
    std::vector<int> wtop;   // elimination schedules of the wide tiles
    for (int ti : torder) {
        const TileType &tt = e->types[ti];
        const std::vector<int> &m = members[ti];
        const bool w = tt.wide != 0;
        const size_t per = w ? 1 : LANES;   // neurons per tile
        for (size_t k = 0; k < m.size(); k += per) {
            Tile t{};
            t.type = ti;
            t.nlanes = (int)std::min<size_t>(per, m.size() - k);
            t.fld = e->rows_fld; e->rows_fld += rows_of(tt.nfields, w);
            t.ints = e->rows_int; e->rows_int += rows_of(tt.nints, w);
            t.pools = e->rows_pool; e->rows_pool += rows_of(tt.npools, w);
            t.giv = e->rows_giv; e->rows_giv += rows_of(tt.ngiv, w);
            t.vm = e->rows_vm; e->rows_vm += rows_of(tt.nslots, w);
            t.topo = e->rows_topo; e->rows_topo += rows_of(tt.nslots, w);
            t.syn = e->rows_syn; e->rows_syn += (int64_t)tt.nsyn * e->ring_len;
            t.scr = e->rows_scr; e->rows_scr += rows_of(tt.nscratch, w);
            t.rav = e->rows_rav; e->rows_rav += rows_of(tt.nrav, w);
            t.itot = e->rows_itot; e->rows_itot += rows_of(tt.nitot, w);
            t.first_neuron = gneuron;
            gneuron += LANES;
            if (w) {
                std::vector<int> sched;
                wide_schedule(dec.neurons[m[k]].parent, sched);
                t.wtop = (int64_t)wtop.size();
                wtop.insert(wtop.end(), sched.begin(), sched.end());
            }
            for (int l = 0; l < t.nlanes; ++l) {
                e->neuron_tile[m[k + l]] = (int)e->tiles.size();
                e->neuron_lane[m[k + l]] = l;
            }
            e->tiles.push_back(t);
        }
    }
    // ---- host images of the device arrays ----
    const size_t L = LANES;
    std::vector<double> P(e->rows_fld * L, 0.0), V(e->rows_vm * L, 0.0), C(e->rows_pool * L, 0.0),
        A(e->rows_topo * L, 0.0), B(e->rows_topo * L, 0.0), Cb(e->rows_topo * L, 0.0);
    std::vector<int> I(e->rows_int * L, 0), par(e->rows_topo * L, -1);
    bool any_stack = false;
    for (const TileType &tt : e->types) any_stack = any_stack || tt.stack;
    std::vector<int> LT(any_stack ? e->rows_topo * L : 1, 0);
    std::vector<double> RV(std::max<int64_t>(e->rows_rav, 1) * L, 0.0);
    // padding lanes: a passive row that solves to zero and never spikes
    for (const Tile &t : e->tiles) {
        const TileType &tt = e->types[t.type];
        if (tt.wide) continue;
        for (int l = t.nlanes; l < LANES; ++l) {
            for (int f = 0; f < tt.nfields; ++f) P[(t.fld + f) * L + l] = 1.0;
            for (int s = 0; s < tt.nslots; ++s) V[(t.vm + s) * L + l] = 0.0;
        }
    }
    // synapse weights per synchan (must be uniform per target synchan)
    std::unordered_map<int64_t, double> wdt;  // key: global neuron * 4096 + syn row
    for (int i = 0; i < nneu; ++i) {
        const Neuron &N = dec.neurons[i];
        const Tile &t = e->tiles[e->neuron_tile[i]];
        const int l = e->neuron_lane[i];
        const bool w = e->types[t.type].wide != 0;
        const int64_t vbase = d->vm_start[N.solver] + N.row0;
        for (int s = 0; s < N.nrows; ++s) {
            V[at(t.vm, s, l, w)] = d->vm[vbase + s];
            par[at(t.topo, s, l, w)] = N.parent[s];
            A[at(t.topo, s, l, w)] = N.A[s];
            B[at(t.topo, s, l, w)] = N.B[s];
            Cb[at(t.topo, s, l, w)] = N.C[s];
        }
        if (e->types[t.type].stack) {
            std::vector<int> fl;
            int cap = 0;
            stack_plan(N.parent, fl, cap);
            const int nst = e->types[t.type].nstatic;
            std::vector<int> sl(N.nrows, 0);
            int fdepth = 0;
            if (e->types[t.type].slots) stack_slots(fl, sl, fdepth);
            for (int s = 0; s < N.nrows; ++s)
                LT[at(t.topo, s, l, false)] = fl[s] | sl[s] | (s < nst && N.parent[s] >= nst ? FL_PD : 0);
        }
        for (size_t f = 0; f < N.fsrc.size(); ++f) P[at(t.fld, f, l, w)] = N.fval[f];
        for (size_t k = 0; k < N.rav.size(); ++k) RV[at(t.rav, k, l, w)] = N.rav[k];
        for (size_t r = 0; r < N.iops.size(); ++r) I[at(t.ints, r, l, w)] = N.ival[r];
        for (size_t p = 0; p < N.pool_conc.size(); ++p)
            C[at(t.pools, p, l, w)] = d->conc[d->conc_start[N.solver] + N.pool_conc[p]];
    }
    // ---- mixed precision: double-float packing of the fields read as df ----
    const bool mixed = e->opt.precision == GBH_PREC_MIXED;
    e->type_df.assign(e->types.size(), std::vector<char>());
    if (mixed) {
        for (size_t ti = 0; ti < e->types.size(); ++ti) e->type_df[ti] = df_fields_of(e->types[ti], prog_pool);
        for (const Tile &t : e->tiles) {
            const std::vector<char> &m = e->type_df[t.type];
            const bool w = e->types[t.type].wide != 0;
            for (int f = 0; f < (int)m.size(); ++f)
                if (m[f])
                    for (int l = 0; l < (w ? 1 : LANES); ++l) P[at(t.fld, f, l, w)] = pack_df(P[at(t.fld, f, l, w)]);
        }
    }
    // ---- synapses: CSR over global neuron index ----
    // Every synapse targets one synchan (a SYN2/SYN3 op of a neuron). A
    // synchan whose synapses all carry one weight keeps weight/dt in its
    // field and counts events; one with different weights gets a SynW
    // descriptor (field value -(1 + index)): a bit per incoming synapse per
    // ring slot, ranked in the order the reference sums the events due in
    // one step -- newest first (synchan.c:239-300 inserts a new event before
    // the pending ones due the same step): by effective delay ascending
    // (later spikes), then by source in the global solver order descending,
    // then by the source's message order descending.
    std::vector<int64_t> out_start(gneuron + 1, 0), out_base, out_mword;
    std::vector<int> out_delay, out_mbit;
    std::vector<SynW> synw;
    std::vector<double> wval;
    int64_t nmask = 0;
    e->spike_pre = false;
    if (e->has_network) {
        // synchan lookup: (solver, op) -> (neuron, syn row)
        std::unordered_map<int64_t, std::pair<int, int>> syn_at;
        for (int i = 0; i < nneu; ++i) {
            const Neuron &N = dec.neurons[i];
            for (size_t r = 0; r < N.syn_op.size(); ++r)
                syn_at[(int64_t)N.solver * (1LL << 32) + N.syn_op[r]] = {i, (int)r};
        }
        std::vector<int> src_neuron(e->nsolvers, -1);
        for (int i = 0; i < nneu; ++i)
            if (dec.neurons[i].spike_op >= 0) src_neuron[dec.neurons[i].solver] = i;
        const int64_t first = remote ? remote->first_solver : 0;   // global index of local solver 0
        // one record per synapse, local ones first (CSR order), then remote
        struct SynRec {
            int tn, srow;             // target neuron and synchan row
            int dl;                   // effective delay (steps)
            int64_t gsrc, k;          // global source index, index in its table
            double wdt;               // weight / dt
            int rank;
        };
        std::vector<SynRec> recs;
        for (int s = 0; s < e->nsolvers && local_syn; ++s) {
            for (int64_t k = syn->src_start[s]; k < syn->src_start[s + 1]; ++k) {
                if (src_neuron[s] < 0)
                    return fail_err(err, GBH_ERR_ARG, "synapse %lld leaves solver %d, which has no spikegen",
                                    (long long)k, s);
                const int ts = syn->target_solver[k];
                if (ts < 0 || ts >= e->nsolvers)
                    return fail_err(err, GBH_ERR_ARG, "synapse %lld targets solver %d", (long long)k, ts);
                auto it = syn_at.find((int64_t)ts * (1LL << 32) + syn->target_op[k]);
                if (it == syn_at.end())
                    return fail_err(err, GBH_ERR_ARG, "synapse %lld: ops[%d] of solver %d is not a SYN2/SYN3 op",
                                    (long long)k, syn->target_op[k], ts);
                const Neuron &SN = dec.neurons[src_neuron[s]];
                int dl = syn->delay_steps[k];
                // a target whose SYN2 op runs before the source's SPIKE op in the
                // same step sees the event one step later (the countdown of this
                // step is already spent)
                if (ts < s || (ts == s && syn->target_op[k] < SN.spike_op)) dl += 1;
                if (dl == 0) e->spike_pre = true;   // acts in the step of the spike
                recs.push_back({it->second.first, it->second.second, dl, first + s, k, syn->weight[k] / e->dt, 0});
            }
        }
        const size_t nlocal = recs.size();
        if (remote && remote->nsources > 0) {
            e->nremote = remote->nsources;
            for (int g = 0; g < remote->nsources; ++g) {
                for (int64_t k = remote->src_start[g]; k < remote->src_start[g + 1]; ++k) {
                    const int ts = remote->target_solver[k];
                    if (ts < 0 || ts >= e->nsolvers)
                        return fail_err(err, GBH_ERR_ARG, "remote synapse %lld targets solver %d", (long long)k, ts);
                    if (remote->delay_steps[k] < 1)
                        return fail_err(err, GBH_ERR_UNSUPPORTED,
                                        "remote synapse %lld acts within the step of the spike: spikes are exchanged "
                                        "between steps", (long long)k);
                    auto it = syn_at.find((int64_t)ts * (1LL << 32) + remote->target_op[k]);
                    if (it == syn_at.end())
                        return fail_err(err, GBH_ERR_ARG,
                                        "remote synapse %lld: ops[%d] of solver %d is not a SYN2/SYN3 op",
                                        (long long)k, remote->target_op[k], ts);
                    recs.push_back({it->second.first, it->second.second, remote->delay_steps[k], (int64_t)g, k,
                                    remote->weight[k] / e->dt, 0});
                }
            }
        }
        // group by target synchan; weights and ranks
        std::map<int64_t, std::vector<size_t>> by_tgt;
        for (size_t r = 0; r < recs.size(); ++r) by_tgt[(int64_t)recs[r].tn * 4096 + recs[r].srow].push_back(r);
        std::vector<int64_t> rec_mword(recs.size(), -1);
        std::vector<int> rec_mbit(recs.size(), 0);
        std::unordered_map<int64_t, double> wfield;   // synchan -> value of its weight field
        for (auto &kv : by_tgt) {
            std::vector<size_t> &v = kv.second;
            bool uniform = true;
            for (size_t r : v) uniform = uniform && recs[r].wdt == recs[v[0]].wdt;
            if (uniform) {
                wfield[kv.first] = recs[v[0]].wdt;
                continue;
            }
            std::sort(v.begin(), v.end(), [&](size_t a, size_t b) {
                const SynRec &x = recs[a], &y = recs[b];
                if (x.dl != y.dl) return x.dl < y.dl;
                if (x.gsrc != y.gsrc) return x.gsrc > y.gsrc;
                return x.k > y.k;
            });
            SynW d{};
            d.nwords = (int)((v.size() + 31) / 32);
            d.mbase = nmask;
            d.wbase = (int64_t)wval.size();
            nmask += (int64_t)d.nwords * e->ring_len;
            for (size_t q = 0; q < v.size(); ++q) {
                wval.push_back(recs[v[q]].wdt);
                rec_mword[v[q]] = d.mbase + (int64_t)(q >> 5);
                rec_mbit[v[q]] = (int)(q & 31) | (d.nwords << 5);
            }
            wfield[kv.first] = -(double)(synw.size() + 1);
            synw.push_back(d);
        }
        const bool weighted = !synw.empty();
        std::vector<std::vector<size_t>> per(gneuron);
        for (size_t r = 0; r < nlocal; ++r) {
            const int s = (int)(recs[r].gsrc - first);
            const int64_t gs = e->tiles[e->neuron_tile[src_neuron[s]]].first_neuron + e->neuron_lane[src_neuron[s]];
            per[gs].push_back(r);
        }
        auto ring_base = [&](const SynRec &x) {
            const Tile &tt = e->tiles[e->neuron_tile[x.tn]];
            return (tt.syn + (int64_t)x.srow * e->ring_len) * LANES + e->neuron_lane[x.tn];
        };
        for (int64_t g = 0; g < gneuron; ++g) {
            out_start[g + 1] = out_start[g] + (int64_t)per[g].size();
            for (size_t r : per[g]) {
                out_base.push_back(ring_base(recs[r]));
                out_delay.push_back(recs[r].dl);
                if (weighted) {
                    out_mword.push_back(rec_mword[r]);
                    out_mbit.push_back(rec_mbit[r]);
                }
            }
        }
        // synapses from remote sources: ring bases, effective delays and rank bits
        if (remote && remote->nsources > 0) {
            std::vector<int64_t> rbase, rmword;
            std::vector<int> rdelay, rmbit;
            for (size_t r = nlocal; r < recs.size(); ++r) {
                rbase.push_back(ring_base(recs[r]));
                rdelay.push_back(recs[r].dl);
                rmword.push_back(rec_mword[r]);
                rmbit.push_back(rec_mbit[r]);
            }
            std::vector<int64_t> rstart(remote->src_start, remote->src_start + remote->nsources + 1);
            if (e->d_rstart.upload(rstart) || e->d_rbase.upload(rbase) || e->d_rdelay.upload(rdelay) ||
                e->d_rbits.alloc(((size_t)remote->nsources + 7) / 8) ||
                (weighted && (e->d_rmword.upload(rmword) || e->d_rmbit.upload(rmbit))))
                return fail_err(err, GBH_ERR_CUDA, "%s", g_last_error);
        }
        for (auto &kv : wfield) {
            const int tn = (int)(kv.first / 4096), srow = (int)(kv.first % 4096);
            const Neuron &N = dec.neurons[tn];
            const Tile &t = e->tiles[e->neuron_tile[tn]];
            for (size_t f = 0; f < N.fsrc.size(); ++f)
                if (N.fsrc[f].kind == FS_WDT && N.fsrc[f].idx == srow)
                    P[at(t.fld, (int64_t)f, e->neuron_lane[tn], e->types[t.type].wide != 0)] = kv.second;
        }
        // spike detection before each step: every neuron with a spike detector
        if (e->spike_pre) {
            std::vector<SpikeSrc> ss;
            for (int i = 0; i < nneu; ++i) {
                const Neuron &N = dec.neurons[i];
                if (N.spike_op < 0) continue;
                const Tile &t = e->tiles[e->neuron_tile[i]];
                const TileType &tt = e->types[t.type];
                const int l = e->neuron_lane[i];
                const bool w = tt.wide != 0;
                int slot = -1, fth = -1, icnt = -1, iref = -1;
                if (!spike_rows(prog_pool, tt, slot, fth, icnt, iref))
                    return fail_err(err, GBH_ERR_ARG, "solver %d: spike detector not found in its program", N.solver);
                SpikeSrc x;
                x.vm = at(t.vm, slot, l, w);
                x.thresh = at(t.fld, fth, l, w);
                x.cnt = at(t.ints, icnt, l, w);
                x.refr = at(t.ints, iref, l, w);
                x.neuron = t.first_neuron + l;
                ss.push_back(x);
            }
            e->nspike_src = (int)ss.size();
            if (e->d_spike_src.upload(ss)) return fail_err(err, GBH_ERR_CUDA, "%s", g_last_error);
        }
    }
    // ---- tables ----
    std::vector<TableGeom> tg;
    std::vector<double> tab64, xy;
    std::vector<float> tab32;
    build_tables(d, tg, tab64, xy);
    tab32.resize(tab64.size());
    for (size_t i = 0; i < tab64.size(); ++i) tab32[i] = (float)tab64[i];
    // double-float entries (value, difference to the next row) for the mixed kernel
    std::vector<float4> tabdf(tab64.size());
    for (int k = 0; k < d->ntables; ++k) {
        TableGeom &g = tg[k];
        const int nc = g.ncols;
        const int64_t rows = nc ? (int64_t)g.xdivs + 2 : 0;   // including the padding row
        for (int64_t r = 0; r < rows; ++r)
            for (int cc = 0; cc < nc; ++cc) {
                const int64_t i = g.tab_off + r * nc + cc;
                const double t0 = tab64[i];
                const double dlt = (r + 1 < rows) ? tab64[i + nc] - t0 : 0.0;
                const float th = (float)t0, dh = (float)dlt;
                tabdf[i] = make_float4(th, (float)(t0 - (double)th), dh, (float)(dlt - (double)dh));
            }
    }
    std::vector<double> stab = dec.stablist;

    // ---- upload ----
    int rc = 0;
    rc |= e->d_tiles.upload(e->tiles);
    rc |= e->d_types.upload(e->types);
    rc |= e->d_prog.upload(prog_pool);
    rc |= e->d_tgeom.upload(tg);
    rc |= e->d_tab64.upload(tab64);
    rc |= e->d_tab32.upload(tab32);
    rc |= e->d_tabdf.upload(tabdf);
    rc |= e->d_xy.upload(xy);
    rc |= e->d_P.upload(P);
    rc |= e->d_V.upload(V);
    rc |= e->d_C.upload(C);
    rc |= e->d_F.upload(std::vector<double>(C.size(), 0.0));
    rc |= e->d_wtop.upload(wtop.empty() ? std::vector<int>(1, 0) : wtop);
    rc |= e->d_RV.upload(RV);
    rc |= e->d_IT.upload(std::vector<double>(std::max<int64_t>(e->rows_itot, 1) * L, 0.0));
    bool any_cd = false;
    for (const TileType &tt : e->types) any_cd = any_cd || tt.has_cd;
    if (any_cd) {   // coresult 0, codiag 1 (hines_conc_init.c:121-126), solve scratch
        rc |= e->d_CR.upload(std::vector<double>(C.size(), 0.0));
        rc |= e->d_CD.upload(std::vector<double>(C.size(), 1.0));
        rc |= e->d_S.upload(std::vector<double>(std::max<int64_t>(e->rows_scr, 1) * L, 0.0));
    }
    rc |= e->d_A.upload(A);
    rc |= e->d_B.upload(B);
    rc |= e->d_Cb.upload(Cb);
    rc |= e->d_I.upload(I);
    rc |= e->d_par.upload(par);
    rc |= e->d_ltop.upload(LT);
    if (any_stack) {
        rc |= e->d_col.alloc(e->rows_topo * L) | e->d_kst.alloc(e->rows_topo * L) | e->d_kri.alloc(e->rows_topo * L);
        rc |= e->d_sgen.upload(std::vector<unsigned>(1, e->sgen_host));
        rc |= e->d_tgen.upload(std::vector<unsigned>(std::max<size_t>(e->tiles.size(), 1), 0u));
        rc |= e->d_kref.upload(std::vector<int>(1, 0));
    }
    rc |= e->d_giv.upload(std::vector<double>(e->rows_giv * L, 0.0));
    rc |= e->d_stab.upload(stab);
    rc |= e->d_ring.upload(std::vector<unsigned>(e->rows_syn * L, 0u));
    rc |= e->d_out_start.upload(out_start);
    rc |= e->d_out_base.upload(out_base);
    rc |= e->d_out_delay.upload(out_delay);
    if (!synw.empty()) {
        rc |= e->d_out_mword.upload(out_mword);
        rc |= e->d_out_mbit.upload(out_mbit);
        rc |= e->d_synw.upload(synw);
        rc |= e->d_wval.upload(wval);
        rc |= e->d_wmask.upload(std::vector<unsigned>(nmask, 0u));
    }
    rc |= e->d_spikes.upload(std::vector<unsigned long long>(gneuron + 1, 0ULL));
    if (e->has_network) rc |= e->d_spiked.upload(std::vector<unsigned>((gneuron + 31) / 32 + 1, 0u));
    rc |= e->d_status.upload(std::vector<int>(1, 0));
    if (rc) return fail_err(err, GBH_ERR_CUDA, "%s", g_last_error);

    // ---- specialised kernels (one per tile type with enough tiles) ----
    std::vector<int> type_t0(e->types.size(), -1), type_t1(e->types.size(), -1);
    for (size_t ti = 0; ti < e->tiles.size(); ++ti) {
        const int ty = e->tiles[ti].type;
        if (type_t0[ty] < 0) type_t0[ty] = (int)ti;
        type_t1[ty] = (int)ti + 1;
    }
    std::vector<int> type_jit(e->types.size(), -1);
    std::vector<char> type_uniform(e->types.size(), 0);
    std::string why;
    const bool jit_on = e->opt.jit >= 0 && jit_available(&why);
    if (!jit_on && e->opt.jit >= 0) e->jit_log = "JIT unavailable: " + why;
    if (jit_on) {
        // types in tile order, largest first
        std::vector<int> cand;
        // the looped forms keep 2 x nslots x 32 rows per warp in shared memory:
        // 4-warp blocks of more than 96 compartments would not fit
        for (int ti : torder)
            if (type_t0[ti] >= 0 && !e->types[ti].wide && !e->types[ti].sym && !e->types[ti].nitot &&
                e->types[ti].nslots <= 96)
                cand.push_back(ti);
        std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) {
            return (type_t1[a] - type_t0[a]) > (type_t1[b] - type_t0[b]);
        });
        const int max_jit = 24;
        if ((int)cand.size() > max_jit) cand.resize(max_jit);
        // residency targets (resident blocks of 4 warps per SM) tried by the autotuner
        // variants: (resident 4-warp blocks per SM, compact form)
        // variants: (warps per block, resident blocks per SM, compact form,
        // unrolled form with its rows in shared memory). Blocks of one or two
        // warps spread the tiles evenly over the SMs (782 4-warp blocks put 6
        // on 22 SMs and 5 on the rest); the shared-rows form is only forced
        // (jit 3): it shrinks the L1 the table gathers hit in
        e->jit_minb.clear();
        e->jit_compact.clear();
        e->jit_smemrows.clear();
        e->jit_warps.clear();
        const int form = e->opt.jit;   // 0 autotuned, 1 unrolled, 2 compact, 3 unrolled with shared rows
        if (e->opt.steps_per_launch > 0 || form > 0) {
            const bool unrolled = form == 0 || form == 1;
            e->jit_minb.push_back(unrolled ? 24 : 6);
            e->jit_compact.push_back(form == 2);
            e->jit_smemrows.push_back(form == 3);
            e->jit_warps.push_back(unrolled ? 1 : 4);
        } else {
            e->jit_minb = {4, 6, 6, 8, 24, 12, 32};
            e->jit_compact = {0, 0, 1, 1, 0, 0, 1};
            e->jit_smemrows = {0, 0, 0, 0, 0, 0, 0};
            e->jit_warps = {4, 4, 4, 4, 1, 2, 1};
        }
        const int nvar = (int)e->jit_minb.size();
        std::vector<std::string> srcs(cand.size() * nvar);
        std::vector<std::vector<int>> upar(cand.size());
        for (size_t c = 0; c < cand.size(); ++c) {
            const int ti = cand[c];
            // is every neuron of this type the same tree?
            bool uni = true;
            std::vector<int> ref;
            for (int i = 0; i < nneu && uni; ++i) {
                if (e->tiles[e->neuron_tile[i]].type != ti) continue;
                if (ref.empty()) ref = dec.neurons[i].parent;
                else if (dec.neurons[i].parent != ref) uni = false;
            }
            if (uni && !ref.empty()) upar[c] = ref;
            for (int vi = 0; vi < nvar; ++vi)
                srcs[c * nvar + vi] = jit_source(e->types[ti], prog_pool, tg[e->types[ti].table_set], mixed, false,
                                                 upar[c].empty() ? nullptr : &upar[c], e->jit_minb[vi],
                                                 e->jit_compact[vi] != 0, e->jit_smemrows[vi] != 0,
                                                 e->jit_warps[vi]);
        }
        int dev = e->opt.device, major = 10, minor = 3;
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
        std::vector<JitKernel> ks(srcs.size());
        std::vector<int> ok(srcs.size(), 0);
        std::vector<std::string> logs(srcs.size());
        std::vector<std::thread> th;
        for (size_t c = 0; c < srcs.size(); ++c)
            th.emplace_back([&, c]() {
                cudaSetDevice(dev);
                if (!srcs[c].empty())
                    ok[c] = jit_compile(srcs[c], !mixed, major, minor, &ks[c], &logs[c]) == 0;
            });
        for (auto &x : th) x.join();
        for (size_t c = 0; c < cand.size(); ++c) {
            bool all = true;
            for (int vi = 0; vi < nvar; ++vi) all = all && ok[c * nvar + vi];
            if (all) {
                type_jit[cand[c]] = (int)e->jits.size();
                type_uniform[cand[c]] = !upar[c].empty();
                std::vector<JitKernel> vars(ks.begin() + c * nvar, ks.begin() + (c + 1) * nvar);
                e->jits.push_back(vars[0]);
                e->jit_var.push_back(vars);
                e->jit_compiled++;
            } else {
                for (int vi = 0; vi < nvar; ++vi) {
                    if (ok[c * nvar + vi]) jit_release(ks[c * nvar + vi]);
                    if (!logs[c * nvar + vi].empty() && e->jit_log.size() < 4000) e->jit_log += logs[c * nvar + vi];
                }
            }
        }
    }
    // ---- launch plan: specialised types alone, the rest bucketed by slot count ----
    size_t t0 = 0;
    while (t0 < e->tiles.size()) {
        const int ty0 = e->tiles[t0].type;
        if (type_jit[ty0] >= 0) {
            const int S = e->types[ty0].nslots;
            Launch L{(int)t0, type_t1[ty0], S, 4};
            L.jit = type_jit[ty0];
            L.uniform = type_uniform[ty0] != 0;
            e->launches.push_back(L);
            t0 = type_t1[ty0];
            continue;
        }
        const int smax = e->types[ty0].nslots;
        size_t t1 = t0;
        if (e->types[ty0].stack) {   // one warp per tile, every size in one launch
            int cap = 1;
            while (t1 < e->tiles.size() && type_jit[e->tiles[t1].type] < 0 && e->types[e->tiles[t1].type].stack) {
                cap = std::max(cap, e->types[e->tiles[t1].type].scap);
                ++t1;
            }
            Launch L{(int)t0, (int)t1, cap, 1};
            L.stack = true;
            for (size_t u = t0; u < t1; ++u) {
                const TileType &tt = e->types[e->tiles[u].type];
                L.split = L.split || (tt.nstatic > 0 && tt.nslots - tt.nstatic <= kSplitRows);
            }
            e->launches.push_back(L);
            t0 = t1;
            continue;
        }
        if (e->types[ty0].wide) {   // one block per neuron
            while (t1 < e->tiles.size() && e->types[e->tiles[t1].type].wide &&
                   e->types[e->tiles[t1].type].nslots * 2 > smax)
                ++t1;
            if (smax * (2 * sizeof(double) + 4 * sizeof(int)) > 200 * 1024)
                return fail_err(err, GBH_ERR_UNSUPPORTED, "neuron with %d compartments exceeds the shared memory",
                                smax);
            Launch L{(int)t0, (int)t1, smax, 1};
            L.wide = true;
            e->launches.push_back(L);
            t0 = t1;
            continue;
        }
        while (t1 < e->tiles.size() && type_jit[e->tiles[t1].type] < 0 && !e->types[e->tiles[t1].type].wide &&
               e->types[e->tiles[t1].type].nslots * 2 > smax)
            ++t1;
        const int per_warp = 2 * smax * LANES * (int)sizeof(double);
        int warps = e->opt.warps_per_block > 0 ? std::min(e->opt.warps_per_block, 4) : 4;
        warps = std::max(1, std::min(warps, kSmemPerBlock / per_warp));
        if (per_warp > 200 * 1024)
            return fail_err(err, GBH_ERR_UNSUPPORTED, "neuron with %d compartments exceeds the shared-memory sweep",
                            smax);
        e->launches.push_back({(int)t0, (int)t1, smax, warps});
        t0 = t1;
    }
    return GBH_OK;
}

DevView view_of(gbh_engine *e)
{
    DevView v{};
    v.tiles = e->d_tiles.p;
    v.types = e->d_types.p;
    v.prog = e->d_prog.p;
    v.tgeom = e->d_tgeom.p;
    v.tab64 = e->d_tab64.p;
    v.tab32 = e->d_tab32.p;
    v.tabdf = e->d_tabdf.p;
    v.xyvals = e->d_xy.p;
    v.P = e->d_P.p;
    v.I = e->d_I.p;
    v.V = e->d_V.p;
    v.C = e->d_C.p;
    v.F = e->d_F.p;
    v.wtop = e->d_wtop.p;
    v.RV = e->d_RV.p;
    v.IT = e->d_IT.p;
    v.CR = e->d_CR.p;
    v.CD = e->d_CD.p;
    v.S = e->d_S.p;
    v.parent = e->d_par.p;
    v.ltop = e->d_ltop.p;
    v.col = e->d_col.p;
    v.kst = e->d_kst.p;
    v.kri = e->d_kri.p;
    v.sgen = e->d_sgen.p;
    v.tgen = e->d_tgen.p;
    v.kref = e->d_kref.p;
    v.A = e->d_A.p;
    v.B = e->d_B.p;
    v.Cb = e->d_Cb.p;
    v.giv = e->d_giv.p;
    v.ring = e->d_ring.p;
    v.ring_len = e->ring_len;
    v.syn_out_start = e->d_out_start.p;
    v.syn_out_base = e->d_out_base.p;
    v.syn_out_delay = e->d_out_delay.p;
    v.syn_out_mword = e->d_out_mword.p;
    v.syn_out_mbit = e->d_out_mbit.p;
    v.wmask = e->d_wmask.p;
    v.synw = e->d_synw.p;
    v.wval = e->d_wval.p;
    v.spike_pre = e->spike_pre ? 1 : 0;
    v.spikes = e->d_spikes.p;
    v.spiked = e->has_network ? e->d_spiked.p : nullptr;
    v.stablist = e->d_stab.p;
    v.status = e->d_status.p;
    v.dt = e->dt;
    return v;
}

int launch_one(gbh_engine *e, const DevView &v, const Launch &L, int k, long long step, bool mixed,
               bool giv, cudaStream_t st)
{
    if (L.jit >= 0 && !giv) {
        // rows in shared-memory columns
        const bool cols = !L.uniform || e->jit_compact[e->jit_choice] || e->jit_smemrows[e->jit_choice];
        const int warps = e->jit_warps[e->jit_choice];
        const size_t smem = cols ? (size_t)warps * 2 * L.smax * LANES * sizeof(double) : 0;
        const cudaError_t je = jit_launch(e->jits[L.jit], v, L.tile0, L.tile1, L.smax, warps, k, step, smem, st);
        if (je != cudaSuccess) {
            set_last("specialised kernel launch failed: %s", cudaGetErrorString(je));
            return GBH_ERR_CUDA;
        }
        e->stats.launches++;
        return GBH_OK;
    }
    cudaError_t ce;
    if (L.stack)
        ce = mixed ? launch_mixed_stack(v, L.tile0, L.tile1, L.smax, k, step, giv, L.split, st)
                   : launch_fp64_stack(v, L.tile0, L.tile1, L.smax, k, step, giv, L.split, st);
    else if (L.wide)
        ce = mixed ? launch_mixed_wide(v, L.tile0, L.tile1, L.smax, k, step, giv, st)
                   : launch_fp64_wide(v, L.tile0, L.tile1, L.smax, k, step, giv, st);
    else
        ce = mixed ? launch_mixed(v, L.tile0, L.tile1, L.smax, L.warps, k, step, giv, st)
                   : launch_fp64(v, L.tile0, L.tile1, L.smax, L.warps, k, step, giv, st);
    if (ce != cudaSuccess) {
        set_last("kernel launch failed: %s", cudaGetErrorString(ce));
        return GBH_ERR_CUDA;
    }
    e->stats.launches++;
    return GBH_OK;
}

// Issues nsteps steps of every launch group, numbered from step0 (absolute,
// or relative to *v.step_dev). With several groups each runs on a side
// stream: groups share no data within a step and, without synapses, none
// across steps, so each group runs its whole span alone; with synapses the
// side streams are joined back into st after every step (events cross
// tiles). giv_last: the last step alone, recording givals.
int issue_steps(gbh_engine *e, const DevView &v, int nsteps, long long step0, bool giv_last, cudaStream_t st,
                int64_t *kernels)
{
    const bool mixed = e->opt.precision == GBH_PREC_MIXED;
    const int nl = (int)e->launches.size();
    const int ns = (int)e->side.size();
    const int plain = giv_last ? nsteps - 1 : nsteps;
    auto spikes = [&](long long step, cudaStream_t s) {   // spike detection before the step
        if (!e->spike_pre) return GBH_OK;
        const int rc = launch_spikes(e, v, step, s);
        if (!rc && kernels) ++*kernels;
        return rc;
    };
    if (nl <= 1 || ns == 0) {
        for (int done = 0; done < plain;) {
            const int k = e->spike_pre ? 1 : std::min(e->steps_per_launch, plain - done);
            if (spikes(step0 + done, st)) return GBH_ERR_CUDA;
            for (const Launch &L : e->launches) {
                const int rc = launch_one(e, v, L, k, step0 + done, mixed, false, st);
                if (rc) return rc;
                if (kernels) ++*kernels;
            }
            done += k;
        }
    } else {
        const int span = e->has_network ? 1 : std::max(plain, 1);
        for (int done = 0; done < plain; done += span) {
            const int n = std::min(span, plain - done);
            if (spikes(step0 + done, st)) return GBH_ERR_CUDA;
            CK(cudaEventRecord(e->ev_fork, st));
            for (int i = 0; i < ns; ++i) CK(cudaStreamWaitEvent(e->side[i], e->ev_fork, 0));
            for (int li = 0; li < nl; ++li) {
                const Launch &L = e->launches[li];
                cudaStream_t s = e->side[li % ns];
                for (int d = 0; d < n;) {
                    const int k = std::min(e->steps_per_launch, n - d);
                    const int rc = launch_one(e, v, L, k, step0 + done + d, mixed, false, s);
                    if (rc) return rc;
                    if (kernels) ++*kernels;
                    d += k;
                }
            }
            for (int i = 0; i < ns; ++i) {
                CK(cudaEventRecord(e->ev_join[i], e->side[i]));
                CK(cudaStreamWaitEvent(st, e->ev_join[i], 0));
            }
        }
    }
    if (giv_last && nsteps > 0) {
        if (spikes(step0 + nsteps - 1, st)) return GBH_ERR_CUDA;
        for (const Launch &L : e->launches) {
            const int rc = launch_one(e, v, L, 1, step0 + nsteps - 1, mixed, true, st);
            if (rc) return rc;
            if (kernels) ++*kernels;
        }
    }
    return GBH_OK;
}

__global__ void k_set_step(long long *s, long long v) { *s = v; }
__global__ void k_add_step(long long *s, long long n) { *s += n; }

void drop_graphs(gbh_engine *e)
{
    for (auto &g : e->graphs) cudaGraphExecDestroy(g.exec);
    e->graphs.clear();
}

// The launch sequence of nsteps steps captured once as a CUDA graph and
// replayed: kernels take their step number from the device counter d_step,
// which the graph's last node advances, so one graph serves every start step.
int run_graph(gbh_engine *e, int nsteps, cudaStream_t st)
{
    gbh_engine::Graph *g = nullptr;
    for (auto &x : e->graphs)
        if (x.nsteps == nsteps && x.spl == e->steps_per_launch && x.variant == e->jit_choice) g = &x;
    if (!g) {
        if (!e->cap_stream) CK(cudaStreamCreateWithFlags(&e->cap_stream, cudaStreamNonBlocking));
        DevView v = view_of(e);
        v.step_dev = e->d_step.p;
        const int64_t launches0 = e->stats.launches;
        CK(cudaStreamBeginCapture(e->cap_stream, cudaStreamCaptureModeRelaxed));
        int64_t kernels = 0;
        const int rc = issue_steps(e, v, nsteps, 0, false, e->cap_stream, &kernels);
        k_add_step<<<1, 1, 0, e->cap_stream>>>(e->d_step.p, nsteps);
        ++kernels;
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(e->cap_stream, &graph);
        e->stats.launches = launches0;
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess) {
            set_last("graph capture failed: %s", cudaGetErrorString(ce));
            return GBH_ERR_CUDA;
        }
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            set_last("graph instantiation failed: %s", cudaGetErrorString(ie));
            return GBH_ERR_CUDA;
        }
        e->graphs.push_back({nsteps, e->steps_per_launch, e->jit_choice, exec, kernels});
        g = &e->graphs.back();
    }
    if (!e->dstep_valid) {
        k_set_step<<<1, 1, 0, st>>>(e->d_step.p, e->step);
        CK(cudaGetLastError());
        e->dstep_valid = true;
    }
    CK(cudaGraphLaunch(g->exec, st));
    e->step += nsteps;
    e->stats.launches += g->kernels;
    return GBH_OK;
}

// Networks: K steps per cooperative launch of the interpreting kernel over
// every tile, a grid barrier between steps (events cross tiles).
int run_coop(gbh_engine *e, int nsteps, cudaStream_t st)
{
    DevView v = view_of(e);
    v.gbar = e->d_gbar.p;
    const bool mixed = e->opt.precision == GBH_PREC_MIXED;
    int smax = 1;
    for (const TileType &tt : e->types) smax = std::max(smax, tt.nslots);
    for (int done = 0; done < nsteps;) {
        const int k = std::min(e->net_spl, nsteps - done);
        CK(cudaMemsetAsync(e->d_gbar.p, 0, 3 * sizeof(unsigned), st));
        const cudaError_t ce = mixed ? launch_mixed_coop(v, (int)e->tiles.size(), smax, k, e->step, st)
                                     : launch_fp64_coop(v, (int)e->tiles.size(), smax, k, e->step, st);
        if (ce != cudaSuccess) {
            set_last("cooperative launch failed: %s", cudaGetErrorString(ce));
            return GBH_ERR_CUDA;
        }
        e->stats.launches++;
        e->step += k;
        done += k;
    }
    return GBH_OK;
}

__global__ void k_bump(unsigned *g) { *g += 1u; }

// The stack tiles' kept factors are redone at their next launch (a field
// they come from may have changed).
int stack_invalidate(gbh_engine *e, cudaStream_t st)
{
    if (!e->d_sgen.p) return GBH_OK;
    k_bump<<<1, 1, 0, st>>>(e->d_sgen.p);
    CK(cudaGetLastError());
    return GBH_OK;
}

int run_steps(gbh_engine *e, int nsteps, cudaStream_t st)
{
    if (e->stack_input_d) {   // inputs write a static row's diagonal term
        const int rci = stack_invalidate(e, st);
        if (rci) return rci;
    }
    if (e->net_coop && !e->givals_enabled && e->nremote == 0) {
        e->dstep_valid = false;
        return run_coop(e, nsteps, st);
    }
    if (e->opt.use_graph && !e->givals_enabled) return run_graph(e, nsteps, st);
    e->dstep_valid = false;   // the launches below carry absolute step numbers
    const DevView v = view_of(e);
    const int rc = issue_steps(e, v, nsteps, e->step, e->givals_enabled, st, nullptr);
    if (rc) return rc;
    e->step += nsteps;
    if (e->givals_enabled) e->givals_valid = true;
    return GBH_OK;
}

}  // namespace

int autotune_trials(gbh_engine *e);

// Autotuner: times trial steps for every (kernel variant, steps per launch)
// candidate on the live engine, saving the mutable state first and restoring
// it after each trial, and keeps the fastest pair. Results are unaffected.
int autotune(gbh_engine *e)
{
    const int use_graph = e->opt.use_graph;
    e->opt.use_graph = 0;   // trials time plain launches; graphs are captured afterwards
    const int rc_t = autotune_trials(e);
    e->opt.use_graph = use_graph;
    drop_graphs(e);
    e->dstep_valid = false;
    // the trials' kernels kept the static rows' factors with their own
    // arithmetic: the chosen kernels keep theirs at their first launch
    if (rc_t == GBH_OK && stack_invalidate(e, e->stream)) return GBH_ERR_CUDA;
    return rc_t;
}

int autotune_trials(gbh_engine *e)
{
    std::vector<int> spls;
    if (e->has_network) spls = {1};
    else spls = {16, 64, 256};
    const int nvar = e->jit_var.empty() ? 1 : (int)e->jit_var[0].size();
    if ((int)spls.size() * nvar <= 1) {
        e->steps_per_launch = spls[0];
        return GBH_OK;
    }
    struct Save { void *dst; const void *src; size_t bytes; };
    std::vector<Save> saves;
    auto keep = [&](void *p, size_t bytes) {
        if (!p || !bytes) return GBH_OK;
        void *b = nullptr;
        if (cudaMalloc(&b, bytes) != cudaSuccess) return GBH_ERR_CUDA;
        saves.push_back({b, p, bytes});
        return GBH_OK;
    };
    int rc = 0;
    rc |= keep(e->d_P.p, e->d_P.n * sizeof(double));
    rc |= keep(e->d_V.p, e->d_V.n * sizeof(double));
    rc |= keep(e->d_C.p, e->d_C.n * sizeof(double));
    rc |= keep(e->d_CR.p, e->d_CR.n * sizeof(double));
    rc |= keep(e->d_CD.p, e->d_CD.n * sizeof(double));
    rc |= keep(e->d_RV.p, e->d_RV.n * sizeof(double));
    rc |= keep(e->d_I.p, e->d_I.n * sizeof(int));
    rc |= keep(e->d_ring.p, e->d_ring.n * sizeof(unsigned));
    rc |= keep(e->d_spikes.p, e->d_spikes.n * sizeof(unsigned long long));
    if (rc) {
        for (Save &s : saves) cudaFree(s.dst);
        return GBH_ERR_CUDA;
    }
    for (Save &s : saves) CK(cudaMemcpy(s.dst, s.src, s.bytes, cudaMemcpyDeviceToDevice));
    double best = 1e300;
    int best_v = 0, best_s = spls[0];
    for (int vi = 0; vi < nvar; ++vi) {
        for (size_t k = 0; k < e->jits.size(); ++k) e->jits[k] = e->jit_var[k][vi];
        e->jit_choice = vi;   // launch_one sizes the shared memory of the variant in use
        for (int spl : spls) {
            e->steps_per_launch = spl;
            const int steps = std::max(2 * spl, 128);
            int rc_t = run_steps(e, 8, e->stream);   // warm caches and clocks
            CK(cudaEventRecord(e->ev0, e->stream));
            if (rc_t == GBH_OK) rc_t = run_steps(e, steps, e->stream);
            CK(cudaEventRecord(e->ev1, e->stream));
            CK(cudaEventSynchronize(e->ev1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
            // a variant that cannot launch here (resources) never wins
            const double per = rc_t == GBH_OK ? ms / steps : 1e300;
            if (rc_t != GBH_OK) cudaGetLastError();
            if (getenv("GBH_VERBOSE") && !e->jit_minb.empty())
                fprintf(stderr, "gbhsolve: trial %d warps x min blocks %d, form %d, %d steps/launch: %.2f us/step\n",
                        e->jit_warps[vi], e->jit_minb[vi], e->jit_compact[vi] ? 1 : e->jit_smemrows[vi] ? 2 : 0, spl,
                        per * 1e3);
            if (per < best) { best = per; best_v = vi; best_s = spl; }
            for (Save &s : saves) CK(cudaMemcpy((void *)s.src, s.dst, s.bytes, cudaMemcpyDeviceToDevice));
        }
    }
    // networks: the cooperative multi-step launch against the best per-step plan
    bool any_wide = false;
    for (const TileType &tt : e->types) any_wide = any_wide || tt.wide;
    if (e->has_network && e->nremote == 0 && e->d_gbar.p && !any_wide && !e->spike_pre) {
        for (size_t k = 0; k < e->jits.size(); ++k) e->jits[k] = e->jit_var[k][best_v];
        e->jit_choice = best_v;
        e->steps_per_launch = best_s;
        int coop_k = 0;
        for (int K : {16, 64}) {
            e->net_coop = true;
            e->net_spl = K;
            const int steps = std::max(2 * K, 128);   // the same length as the per-step trials
            int rc_c = run_steps(e, 8, e->stream);
            if (rc_c == GBH_OK) {
                CK(cudaEventRecord(e->ev0, e->stream));
                rc_c = run_steps(e, steps, e->stream);
                CK(cudaEventRecord(e->ev1, e->stream));
            }
            const cudaError_t se = cudaEventSynchronize(e->ev1);
            float ms = 0.f;
            if (rc_c == GBH_OK && se == cudaSuccess && cudaEventElapsedTime(&ms, e->ev0, e->ev1) == cudaSuccess) {
                const double per = ms / steps;
                if (per < best) { best = per; coop_k = K; }
            } else {
                cudaGetLastError();   // e.g. too many tiles to be resident at once: keep per-step launches
            }
            e->net_coop = false;
            for (Save &s : saves) CK(cudaMemcpy((void *)s.src, s.dst, s.bytes, cudaMemcpyDeviceToDevice));
        }
        int status = 0;
        CK(cudaMemcpy(&status, e->d_status.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (status & ST_BARRIER) {   // a barrier ran out: keep per-step launches
            coop_k = 0;
            status &= ~ST_BARRIER;
            CK(cudaMemcpy(e->d_status.p, &status, sizeof(int), cudaMemcpyHostToDevice));
        }
        if (coop_k) {
            e->net_coop = true;
            e->net_spl = coop_k;
        }
    }
    for (Save &s : saves) cudaFree(s.dst);
    if (e->d_spiked.p) CK(cudaMemset(e->d_spiked.p, 0, e->d_spiked.n * sizeof(unsigned)));   // trial spikes
    if (e->rows_itot) CK(cudaMemset(e->d_IT.p, 0, e->d_IT.n * sizeof(double)));   // trial itotal sums
    for (size_t k = 0; k < e->jits.size(); ++k) e->jits[k] = e->jit_var[k][best_v];
    e->jit_choice = best_v;
    e->steps_per_launch = best_s;
    e->step = 0;
    e->stats.launches = 0;
    return GBH_OK;
}

// Internal: the step loop of run_steps with the flux scratch supplied by the
// caller (used by gbh_run_noalloc). Reports the flux elements the engine needs,
// the engine's own flux rows, device and stream.
int64_t gbh_internal_flux_elems(const gbh_engine *e) { return e->rows_pool * (int64_t)LANES; }
double *gbh_internal_flux_rows(const gbh_engine *e) { return e->d_F.p; }
int gbh_internal_device(const gbh_engine *e) { return e->opt.device; }
cudaStream_t gbh_internal_stream(const gbh_engine *e) { return e->stream; }

int gbh_internal_run_with_flux(gbh_engine *e, int nsteps, cudaStream_t st, double *flux)
{
    e->dstep_valid = false;
    DevView v = view_of(e);
    v.F = flux;
    const int rc = issue_steps(e, v, nsteps, e->step, e->givals_enabled, st, nullptr);
    if (rc) return rc;
    e->step += nsteps;
    e->stats.steps += nsteps;
    if (e->givals_enabled) e->givals_valid = true;
    return GBH_OK;
}

constexpr int64_t kPackedFlag = 1LL << 62;   // input target holds a packed double-float
constexpr int64_t kFluxFlag = 1LL << 61;     // input target is a flux row (F), not a field (P)
constexpr int64_t kAddFlag = 1LL << 60;      // input adds v*sa*sb when v > VTINY (SYN2 messages)
constexpr int64_t kAddrMask = (1LL << 60) - 1;

// Registered inputs grouped by target: each thread applies the inputs of one
// target in registration order, as h_in_msgs walks its list
// (hines_msgs.c:351-405): INJECT/BASE/THRESH set a chip value, SYN2 adds
// X*stablist[nop+3] (*dt for ACTIVATION messages) when X > VTINY, FLUX sets
// the flux of a concentration.
struct InPlan {
    const int64_t *start;   // [ntgt+1] items of each target
    const int *item;        // input index of each item
    const double *sa, *sb;  // factors of an adding item
    const int64_t *addr;    // target address and flags
    int ntgt;
};

__device__ __forceinline__ void apply_inputs(const InPlan &pl, int t, const double *vals, double *P, double *F)
{
    const int64_t a = pl.addr[t];
    double *dst = (a & kFluxFlag) ? &F[a & kAddrMask] : &P[a & kAddrMask];
    const bool packed = (a & kPackedFlag) != 0;
    double x;
    if (packed) {
        const float2 f = *reinterpret_cast<const float2 *>(dst);
        x = (double)f.x + (double)f.y;
    } else {
        x = *dst;
    }
    for (int64_t k = pl.start[t]; k < pl.start[t + 1]; ++k) {
        const double v = vals[pl.item[k]];
        if (a & kAddFlag) {
            // explicit roundings: no multiply-add contraction, as the host does it
            if (v > 1.0e-10) x = __dadd_rn(x, __dmul_rn(__dmul_rn(v, pl.sa[k]), pl.sb[k]));
        } else {
            x = v;
        }
    }
    if (packed) {
        const float hi = __double2float_rn(x);
        const float lo = __double2float_rn(x - (double)hi);
        *reinterpret_cast<float2 *>(dst) = make_float2(hi, lo);
    } else {
        *dst = x;
    }
}

__global__ void k_scatter_inputs(const double *vals, InPlan pl, double *P, double *F)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < pl.ntgt) apply_inputs(pl, t, vals, P, F);
}

// Between two steps: the outputs of the step just run (gather, n_out) and
// the inputs of the next (one thread per input target) in one launch.
__global__ void k_io(const double *V, const int64_t *out_addr, int n_out, double *out, const double *in_vals,
                     InPlan pl, double *P, double *F)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_out) out[i] = V[out_addr[i]];
    if (in_vals && i < pl.ntgt) apply_inputs(pl, i, in_vals, P, F);
}

// Events of remote spikes: source i spiked during step `step`; each of its
// synapses adds one event to its target synchan's ring slot for the step
// the spike acts in.
__global__ void k_deliver_remote(const unsigned char *bits, int n, const int64_t *start, const int64_t *base,
                                 const int *delay, const int64_t *mword, const int *mbit, unsigned *ring,
                                 unsigned *wmask, int ring_len, long long step)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !(bits[i >> 3] & (1u << (i & 7)))) return;
    for (int64_t k = start[i]; k < start[i + 1]; ++k)
        put_event(ring, ring_len, wmask, base[k], delay[k], mword ? mword[k] : -1, mbit ? mbit[k] : 0, step);
}

// Spike detection of every neuron with a spike detector, before the step's
// channel programs (networks whose synapses can act in the step of the
// spike): SPIKE_OP reads only the compartment's Vm at the start of the step
// and the neuron's own counters, so the step kernels then skip it.
__global__ void k_spikes(DevView v, const SpikeSrc *src, int n, long long step0)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long step = (v.step_dev ? *v.step_dev : 0) + step0;
    const SpikeSrc x = src[i];
    v.I[x.cnt] = spike_op(v, v.V[x.vm], v.P[x.thresh], v.I[x.cnt], v.I[x.refr], true, x.neuron, step);
}

int launch_spikes(gbh_engine *e, const DevView &v, long long step, cudaStream_t st)
{
    const int threads = 128, blocks = (e->nspike_src + threads - 1) / threads;
    if (blocks > 0) k_spikes<<<blocks, threads, 0, st>>>(v, e->d_spike_src.p, e->nspike_src, step);
    const cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) {
        set_last("spike detection launch failed: %s", cudaGetErrorString(ce));
        return GBH_ERR_CUDA;
    }
    e->stats.launches++;
    return GBH_OK;
}

__global__ void k_gather_outputs(const double *V, const int64_t *addr, int n, double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = V[addr[i]];
}

extern "C" {

const char *gbh_last_error(void) { return g_last_error; }

// Per-tile CSR of (offset within the tile's block, index) pairs.
int upload_tile_lists(gbh_engine *e, std::vector<std::vector<std::pair<int, int>>> &per_tile, DBuf<int> &start,
                      DBuf<int> &off, DBuf<int> &idx)
{
    std::vector<int> st(per_tile.size() + 1, 0), o, ix;
    for (size_t t = 0; t < per_tile.size(); ++t) {
        for (auto &x : per_tile[t]) {
            o.push_back(x.first);
            ix.push_back(x.second);
        }
        st[t + 1] = (int)o.size();
    }
    if (o.empty()) {
        o.push_back(0);
        ix.push_back(0);
    }
    start.release(); off.release(); idx.release();
    if (start.upload(st) || off.upload(o) || idx.upload(ix)) return GBH_ERR_CUDA;
    (void)e;
    return GBH_OK;
}

InPlan in_plan(const gbh_engine *e)
{
    InPlan pl;
    pl.start = e->d_in_start.p;
    pl.item = e->d_in_item.p;
    pl.sa = e->d_in_sa.p;
    pl.sb = e->d_in_sb.p;
    pl.addr = e->d_in_addr.p;
    pl.ntgt = e->n_tgt;
    return pl;
}

int gbh_register_inputs_typed(gbh_engine *e, int n, const int *solver, const int *kind, const int64_t *index,
                              const double *sa, const double *sb)
{
    if (!e || n < 0 || (n && (!solver || !index))) return GBH_ERR_ARG;
    // target address (with flags) of every input; inputs sharing a target are
    // applied in registration order by one thread
    std::vector<std::vector<int64_t>> addrs(n);
    std::unordered_map<int64_t, std::vector<int>> want_chip, want_conc;
    for (int i = 0; i < n; ++i) {
        if (solver[i] < 0 || solver[i] >= e->nsolvers) return GBH_ERR_ARG;
        const int k = kind ? kind[i] : GBH_IN_SET;
        if (k != GBH_IN_SET && k != GBH_IN_ADD && k != GBH_IN_FLUX) {
            set_last("input %d: unknown kind %d", i, k);
            return GBH_ERR_ARG;
        }
        if (k == GBH_IN_FLUX) want_conc[e->conc_start[solver[i]] + index[i]].push_back(i);
        else want_chip[e->chip_start[solver[i]] + index[i]].push_back(i);
    }
    bool kfield_input = false;   // an input writes a static row's rhs fields
    for (size_t q = 0; q < e->dec.neurons.size(); ++q) {
        const Neuron &N = e->dec.neurons[q];
        const Tile &t = e->tiles[e->neuron_tile[q]];
        const int l = e->neuron_lane[q];
        for (size_t f = 0; f < N.fsrc.size(); ++f) {
            if (N.fsrc[f].kind != FS_CHIP) continue;
            auto it = want_chip.find(e->chip_start[N.solver] + N.fsrc[f].idx);
            if (it == want_chip.end()) continue;
            const bool packed = !e->type_df[t.type].empty() && e->type_df[t.type][f];
            if ((size_t)t.type < e->stack_dfield.size() && !e->stack_dfield[t.type].empty() &&
                e->stack_dfield[t.type][f])
                e->stack_input_d = true;
            if ((size_t)t.type < e->stack_kfield.size() && !e->stack_kfield[t.type].empty() &&
                e->stack_kfield[t.type][f])
                kfield_input = true;
            for (int i : it->second) {
                const bool add = kind && kind[i] == GBH_IN_ADD;
                addrs[i].push_back(at(t.fld, (int64_t)f, l, e->types[t.type].wide != 0) |
                                   (packed ? kPackedFlag : 0) | (add ? kAddFlag : 0));
            }
        }
        for (size_t p = 0; p < N.pool_conc.size(); ++p) {
            auto it = want_conc.find(e->conc_start[N.solver] + N.pool_conc[p]);
            if (it == want_conc.end()) continue;
            for (int i : it->second)
                addrs[i].push_back(at(t.pools, (int64_t)p, l, e->types[t.type].wide != 0) | kFluxFlag);
        }
    }
    // the stack tiles then refresh those terms at every launch, the specialised
    // kernels at every step (2: a diagonal term, every step of theirs a full one)
    if ((kfield_input || e->stack_input_d) && e->d_kref.p) {
        const int kr = e->stack_input_d ? 2 : 1;
        CK(cudaStreamSynchronize(e->stream));
        CK(cudaMemcpy(e->d_kref.p, &kr, sizeof(int), cudaMemcpyHostToDevice));
    }
    std::map<int64_t, std::vector<int>> by_target;   // keyed by address without the add flag
    std::map<int64_t, int64_t> flags;
    for (int i = 0; i < n; ++i) {
        if (addrs[i].empty()) {
            set_last("input %d (solver %d, index %lld) is not read by any compartment program", i, solver[i],
                     (long long)index[i]);
            return GBH_ERR_ARG;
        }
        for (int64_t a : addrs[i]) {
            const int64_t key = a & ~kAddFlag;
            auto f = flags.find(key);
            if (f != flags.end() && (f->second & kAddFlag) != (a & kAddFlag)) {
                set_last("input %d: a target both set and added to", i);
                return GBH_ERR_ARG;
            }
            flags[key] = a;
            by_target[key].push_back(i);
        }
    }
    std::vector<int64_t> start(1, 0), taddr;
    std::vector<int> item;
    std::vector<double> fa, fb;
    for (auto &kv : by_target) {
        taddr.push_back(flags[kv.first]);
        for (int i : kv.second) {
            item.push_back(i);
            fa.push_back(sa ? sa[i] : 1.0);
            fb.push_back(sb ? sb[i] : 1.0);
        }
        start.push_back((int64_t)item.size());
    }
    e->d_in_vals.release(); e->d_in_start.release(); e->d_in_addr.release();
    e->d_in_item.release(); e->d_in_sa.release(); e->d_in_sb.release();
    if (e->d_in_vals.alloc(n) || e->d_in_start.upload(start) || e->d_in_addr.upload(taddr) ||
        e->d_in_item.upload(item) || e->d_in_sa.upload(fa) || e->d_in_sb.upload(fb))
        return GBH_ERR_CUDA;
    e->n_in = n;
    e->n_tgt = (int)taddr.size();
    // the fused form: only set-inputs on lane tiles' inject rows (M_BEGIN's
    // second operand); the last one registered for a row wins, as h_in_msgs
    e->fuse_in = true;
    std::vector<std::vector<std::pair<int, int>>> per_tile(e->tiles.size());
    std::map<std::pair<int, int>, int> last;   // (tile, offset) -> input
    for (size_t q = 0; q < e->dec.neurons.size() && e->fuse_in; ++q) {
        const Neuron &N = e->dec.neurons[q];
        const int ti = e->neuron_tile[q];
        const Tile &t = e->tiles[ti];
        const int l = e->neuron_lane[q];
        std::vector<char> inject(N.fsrc.size(), 0);
        for (size_t pc = 0; pc < N.prog.size();) {
            const int code = N.prog[pc];
            const int m = micro_operands(code);
            if (m < 0) break;
            if (code == M_BEGIN) inject[N.prog[pc + 2]] = 1;
            pc += 1 + m;
        }
        for (size_t f = 0; f < N.fsrc.size(); ++f) {
            if (N.fsrc[f].kind != FS_CHIP) continue;
            auto it = want_chip.find(e->chip_start[N.solver] + N.fsrc[f].idx);
            if (it == want_chip.end()) continue;
            for (int i : it->second) {
                if ((kind && kind[i] != GBH_IN_SET) || !inject[f] || e->types[t.type].wide) {
                    e->fuse_in = false;
                    break;
                }
                const bool packed = !e->type_df[t.type].empty() && e->type_df[t.type][f];
                last[{ti, (int)(f * LANES + l) | (packed ? (1 << 30) : 0)}] = i;
            }
        }
    }
    if (!want_conc.empty()) e->fuse_in = false;
    if (e->fuse_in) {
        for (auto &kv : last) per_tile[kv.first.first].push_back({kv.first.second, kv.second});
        if (upload_tile_lists(e, per_tile, e->d_tin_start, e->d_tin_off, e->d_tin_idx)) return GBH_ERR_CUDA;
    }
    return GBH_OK;
}

int gbh_register_inputs(gbh_engine *e, int n, const int *solver, const int64_t *chip_index)
{
    return gbh_register_inputs_typed(e, n, solver, nullptr, chip_index, nullptr, nullptr);
}

int gbh_set_inputs_async(gbh_engine *e, const double *host_values, void *stream)
{
    if (!e || !host_values) return GBH_ERR_ARG;
    if (e->n_in == 0) return GBH_OK;
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    CK(cudaMemcpyAsync(e->d_in_vals.p, host_values, e->n_in * sizeof(double), cudaMemcpyHostToDevice, st));
    k_scatter_inputs<<<(e->n_tgt + 255) / 256, 256, 0, st>>>(e->d_in_vals.p, in_plan(e), e->d_P.p, e->d_F.p);
    CK(cudaGetLastError());
    return GBH_OK;
}

int gbh_register_outputs(gbh_engine *e, int n, const int *solver, const int *row)
{
    if (!e || n < 0 || (n && (!solver || !row))) return GBH_ERR_ARG;
    // (solver, row) -> neuron: neurons of a solver are contiguous in row order
    std::vector<int64_t> addr(n);
    for (int i = 0; i < n; ++i) {
        const int s = solver[i];
        if (s < 0 || s >= e->nsolvers) return GBH_ERR_ARG;
        int found = -1;
        for (int k = e->dec.solver_first_neuron[s]; k < e->dec.solver_first_neuron[s + 1]; ++k) {
            const Neuron &N = e->dec.neurons[k];
            if (row[i] >= N.row0 && row[i] < N.row0 + N.nrows) { found = k; break; }
        }
        if (found < 0) return GBH_ERR_ARG;
        const Neuron &N = e->dec.neurons[found];
        const Tile &t = e->tiles[e->neuron_tile[found]];
        addr[i] = at(t.vm, row[i] - N.row0, e->neuron_lane[found], e->types[t.type].wide != 0);
    }
    e->d_out_vals.release(); e->d_out_addr.release();
    if (e->d_out_vals.alloc(n) || e->d_out_addr.upload(addr)) return GBH_ERR_CUDA;
    e->n_out = n;
    std::vector<std::vector<std::pair<int, int>>> per_tile(e->tiles.size());
    for (int i = 0; i < n; ++i) {   // the tile of each output, from its address
        for (size_t t = 0; t < e->tiles.size(); ++t) {
            const Tile &tl = e->tiles[t];
            const int64_t rows = rows_of(e->types[tl.type].nslots, e->types[tl.type].wide != 0);
            if (addr[i] >= tl.vm * LANES && addr[i] < (tl.vm + rows) * LANES) {
                per_tile[t].push_back({(int)(addr[i] - tl.vm * LANES), i});
                break;
            }
        }
    }
    if (upload_tile_lists(e, per_tile, e->d_tout_start, e->d_tout_off, e->d_tout_idx)) return GBH_ERR_CUDA;
    return GBH_OK;
}

int gbh_get_outputs_async(gbh_engine *e, double *host_values, void *stream)
{
    if (!e || !host_values) return GBH_ERR_ARG;
    if (e->n_out == 0) return GBH_OK;
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    k_gather_outputs<<<(e->n_out + 255) / 256, 256, 0, st>>>(e->d_V.p, e->d_out_addr.p, e->n_out,
                                                             e->d_out_vals.p);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host_values, e->d_out_vals.p, e->n_out * sizeof(double), cudaMemcpyDeviceToHost, st));
    return GBH_OK;
}

// Issues the deferred output copy of the previous call together with this
// call's input scatter (in_buf < 0: no input).
static int io_between(gbh_engine *e, cudaStream_t st, int in_buf)
{
    const bool out = e->io_pend_host != nullptr;
    const int n_tg = in_buf >= 0 ? e->n_tgt : 0;
    const int n_out = out ? e->n_out : 0;
    const int n = std::max(n_tg, n_out);
    if (n == 0) return GBH_OK;
    k_io<<<(n + 255) / 256, 256, 0, st>>>(e->d_V.p, e->d_out_addr.p, n_out, out ? e->d_io_out[e->io_pend_buf].p : nullptr,
                                          in_buf >= 0 ? e->d_io_in[in_buf].p : nullptr, in_plan(e), e->d_P.p,
                                          e->d_F.p);
    CK(cudaGetLastError());
    if (out) {
        const int pb = e->io_pend_buf;
        CK(cudaEventRecord(e->io_gathered[pb], st));
        CK(cudaStreamWaitEvent(e->io_out_stream, e->io_gathered[pb], 0));
        CK(cudaMemcpyAsync(e->io_pend_host, e->d_io_out[pb].p, e->n_out * sizeof(double), cudaMemcpyDeviceToHost,
                           e->io_out_stream));
        CK(cudaEventRecord(e->io_out_copied[pb], e->io_out_stream));
        e->io_pend_host = nullptr;
    }
    return GBH_OK;
}

int gbh_step_io(gbh_engine *e, const double *host_in, double *host_out, int nsteps, void *stream)
{
    if (!e || nsteps < 0) return GBH_ERR_ARG;
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    if (!e->io_stream || e->io_nin != e->n_in || e->io_nout != e->n_out) {
        const int rc = gbh_io_sync(e);
        if (rc) return rc;
        if (!e->io_stream) {
            CK(cudaStreamCreateWithFlags(&e->io_stream, cudaStreamNonBlocking));
            CK(cudaStreamCreateWithFlags(&e->io_out_stream, cudaStreamNonBlocking));
            for (int b = 0; b < 2; ++b) {
                CK(cudaEventCreateWithFlags(&e->io_in_copied[b], cudaEventDisableTiming));
                CK(cudaEventCreateWithFlags(&e->io_gathered[b], cudaEventDisableTiming));
                CK(cudaEventCreateWithFlags(&e->io_out_copied[b], cudaEventDisableTiming));
            }
        }
        for (int b = 0; b < 2; ++b) {
            e->d_io_in[b].release();
            e->d_io_out[b].release();
            if (e->d_io_in[b].alloc(e->n_in) || e->d_io_out[b].alloc(e->n_out)) return GBH_ERR_CUDA;
        }
        e->io_nin = e->n_in;
        e->io_nout = e->n_out;
        e->io_calls = 0;
    }
    const int b = (int)(e->io_calls & 1);
    // the buffers of the call before last are free once its output copy is done
    if (e->io_calls >= 2) CK(cudaEventSynchronize(e->io_out_copied[b]));
    int in_buf = -1;
    if (e->n_in && host_in) {
        CK(cudaMemcpyAsync(e->d_io_in[b].p, host_in, e->n_in * sizeof(double), cudaMemcpyHostToDevice, e->io_stream));
        CK(cudaEventRecord(e->io_in_copied[b], e->io_stream));
        CK(cudaStreamWaitEvent(st, e->io_in_copied[b], 0));
        in_buf = b;
    }
    int rc = io_between(e, st, in_buf);
    if (rc) return rc;
    if (nsteps > 0) {
        rc = run_steps(e, nsteps, st);
        if (rc) return rc;
    }
    if (e->n_out && host_out) {
        e->io_pend_host = host_out;   // gathered before the next call's steps
        e->io_pend_buf = b;
        e->io_pend_stream = st;
    } else {
        CK(cudaEventRecord(e->io_out_copied[b], st));
    }
    e->io_calls++;
    e->stats.steps += nsteps;
    return GBH_OK;
}

int gbh_run_io(gbh_engine *e, const double *host_in, double *host_out, int nsteps, int block, void *stream)
{
    if (!e || nsteps < 0 || block < 0) return GBH_ERR_ARG;
    if (nsteps == 0) return GBH_OK;
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    int rc = gbh_io_sync(e);   // pipelined gbh_step_io calls complete first
    if (rc) return rc;
    const int n_in = host_in ? (int)e->n_in : 0, n_out = host_out ? (int)e->n_out : 0;
    const int B = std::min(block > 0 ? block : 16, nsteps);
    if (!e->io_stream) {
        CK(cudaStreamCreateWithFlags(&e->io_stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&e->io_out_stream, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            CK(cudaEventCreateWithFlags(&e->io_in_copied[b], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&e->io_gathered[b], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&e->io_out_copied[b], cudaEventDisableTiming));
        }
    }
    if (!e->blk_done[0])
        for (int b = 0; b < 2; ++b) {
            CK(cudaEventCreateWithFlags(&e->blk_in_copied[b], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&e->blk_done[b], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&e->blk_out_copied[b], cudaEventDisableTiming));
        }
    if (B > e->blk_cap || n_in != e->blk_nin || n_out != e->blk_nout) {
        for (int b = 0; b < 2; ++b) {
            CK(cudaEventSynchronize(e->blk_done[b]));
            CK(cudaEventSynchronize(e->blk_out_copied[b]));
            e->d_blk_in[b].release();
            e->d_blk_out[b].release();
            if (e->d_blk_in[b].alloc((size_t)B * n_in) || e->d_blk_out[b].alloc((size_t)B * n_out))
                return GBH_ERR_CUDA;
        }
        e->blk_cap = B;
        e->blk_nin = n_in;
        e->blk_nout = n_out;
    }
    const int nio = std::max(n_in ? e->n_tgt : 0, n_out);
    const InPlan plan = in_plan(e);
    // every launch group specialised (lane tiles), no synapses: the step
    // kernels apply each step's inputs and gather its outputs themselves, and
    // a block of steps runs as multi-step launches
    bool fused = !e->has_network && !e->givals_enabled && !e->net_coop && (n_in == 0 || e->fuse_in) &&
                 !e->launches.empty();
    for (const Launch &L : e->launches) fused = fused && L.jit >= 0 && !L.wide;
    const unsigned grid = (unsigned)((nio + 255) / 256);
    int last = 0;
    for (int s0 = 0, j = 0; s0 < nsteps; s0 += B, ++j) {
        const int nb = std::min(B, nsteps - s0), b = j & 1;
        double *din = e->d_blk_in[b].p, *dout = e->d_blk_out[b].p;
        if (n_in) {
            // staging b is free once the block that used it two blocks ago has stepped
            CK(cudaStreamWaitEvent(e->io_stream, e->blk_done[b], 0));
            CK(cudaMemcpyAsync(din, host_in + (int64_t)s0 * n_in, (size_t)nb * n_in * sizeof(double),
                               cudaMemcpyHostToDevice, e->io_stream));
            CK(cudaEventRecord(e->blk_in_copied[b], e->io_stream));
            CK(cudaStreamWaitEvent(st, e->blk_in_copied[b], 0));
            if (!fused) {
                k_io<<<grid, 256, 0, st>>>(e->d_V.p, e->d_out_addr.p, 0, nullptr, din, plan, e->d_P.p, e->d_F.p);
                CK(cudaGetLastError());
            }
        }
        if (n_out) CK(cudaStreamWaitEvent(st, e->blk_out_copied[b], 0));   // its outputs were copied out
        if (fused) {
            DevView v = view_of(e);
            v.io_in = n_in ? din : nullptr;
            v.io_out = n_out ? dout : nullptr;
            v.io_nin = n_in;
            v.io_nout = n_out;
            v.io_step0 = e->step;
            v.tin_start = e->d_tin_start.p;
            v.tin_off = e->d_tin_off.p;
            v.tin_idx = e->d_tin_idx.p;
            v.tout_start = e->d_tout_start.p;
            v.tout_off = e->d_tout_off.p;
            v.tout_idx = e->d_tout_idx.p;
            e->dstep_valid = false;   // absolute step numbers in the launches
            rc = issue_steps(e, v, nb, e->step, false, st, nullptr);
            if (rc) return rc;
            e->step += nb;
            CK(cudaEventRecord(e->blk_done[b], st));
            if (n_out) {
                CK(cudaStreamWaitEvent(e->io_out_stream, e->blk_done[b], 0));
                CK(cudaMemcpyAsync(host_out + (int64_t)s0 * n_out, dout, (size_t)nb * n_out * sizeof(double),
                                   cudaMemcpyDeviceToHost, e->io_out_stream));
                CK(cudaEventRecord(e->blk_out_copied[b], e->io_out_stream));
            }
            last = b;
            continue;
        }
        for (int k = 0; k < nb; ++k) {
            rc = run_steps(e, 1, st);
            if (rc) return rc;
            // this step's outputs and the next step's inputs, one launch
            const int go = n_out, si = k + 1 < nb ? n_in : 0;
            if (go || si) {
                k_io<<<grid, 256, 0, st>>>(e->d_V.p, e->d_out_addr.p, go, dout + (int64_t)k * n_out,
                                           si ? din + (int64_t)(k + 1) * n_in : nullptr, plan, e->d_P.p, e->d_F.p);
                CK(cudaGetLastError());
            }
        }
        CK(cudaEventRecord(e->blk_done[b], st));
        if (n_out) {
            CK(cudaStreamWaitEvent(e->io_out_stream, e->blk_done[b], 0));
            CK(cudaMemcpyAsync(host_out + (int64_t)s0 * n_out, dout, (size_t)nb * n_out * sizeof(double),
                               cudaMemcpyDeviceToHost, e->io_out_stream));
            CK(cudaEventRecord(e->blk_out_copied[b], e->io_out_stream));
        }
        last = b;
    }
    CK(cudaEventSynchronize(e->blk_done[last]));
    if (n_out) CK(cudaEventSynchronize(e->blk_out_copied[last]));
    e->stats.steps += nsteps;
    return GBH_OK;
}

int gbh_io_sync(gbh_engine *e)
{
    if (!e) return GBH_ERR_ARG;
    if (e->io_pend_host) {
        const int rc = io_between(e, e->io_pend_stream, -1);
        if (rc) return rc;
    }
    if (e->io_stream) CK(cudaStreamSynchronize(e->io_stream));
    if (e->io_out_stream) CK(cudaStreamSynchronize(e->io_out_stream));
    for (int b = 0; b < 2; ++b)
        if (e->io_out_copied[b]) CK(cudaEventSynchronize(e->io_out_copied[b]));
    return GBH_OK;
}

int64_t gbh_jit_source(const gbh_batch_desc *desc, int precision, int type_index, int compact, char *buf,
                       int64_t buflen)
{
    gbh_error err{};
    Decoded dec;
    if (decode_batch(desc, dec, &err)) {
        set_last("%s", err.message);
        return err.code;
    }
    std::map<std::string, int> keys;
    std::vector<TileType> types;
    std::vector<int> prog_pool;
    std::vector<std::vector<int>> parents;
    std::vector<char> uniform;
    for (const Neuron &N : dec.neurons) {
        auto it = keys.find(N.key);
        if (it == keys.end()) {
            TileType tt{};
            tt.nslots = N.nrows;
            tt.nfields = (int)N.fsrc.size();
            tt.nints = (int)N.iops.size();
            tt.npools = (int)N.pool_conc.size();
            tt.ngiv = (int)N.giv_ref.size();
            tt.prog_off = (int)prog_pool.size();
            prog_pool.insert(prog_pool.end(), N.prog.begin(), N.prog.end());
            tt.pool_off = (int)prog_pool.size();
            prog_pool.insert(prog_pool.end(), N.pool_prog.begin(), N.pool_prog.end());
            tt.table_set = N.table_set;
            tt.crank = N.crank;
            tt.chanmode5 = N.c5;
            tt.interp = N.interp;
            tt.has_cd = N.has_cd;
            tt.nscratch = N.nscratch;
            tt.sym = !N.sym.empty();
            tt.nitot = N.nitot;
            keys[N.key] = (int)types.size();
            types.push_back(tt);
            parents.push_back(N.parent);
            uniform.push_back(1);
        } else if (parents[it->second] != N.parent) {
            uniform[it->second] = 0;
        }
    }
    if (type_index < 0 || type_index >= (int)types.size()) return GBH_ERR_ARG;
    {   // the static rows as the engine plans them for a stack-eligible type
        TileType &tt = types[type_index];
        std::vector<int> fl;
        int cap = 0;
        if (!tt.sym && tt.nslots >= kStackMin && stack_plan(parents[type_index], fl, cap) && cap <= kStackCapMax) {
            const std::vector<int> pf = slot_field_ranges(prog_pool, tt);
            while (tt.nstatic < tt.nslots && pf[6 * tt.nstatic + 2] >= 0) ++tt.nstatic;
        }
    }
    std::vector<TableGeom> tg;
    std::vector<double> tab64, xy;
    build_tables(desc, tg, tab64, xy);
    const std::string src = jit_source(types[type_index], prog_pool, tg[types[type_index].table_set],
                                       precision == GBH_PREC_MIXED, false,
                                       uniform[type_index] ? &parents[type_index] : nullptr, 6, compact == 1,
                                       compact == 2);
    if (buf && buflen > 0) {
        const int64_t n = std::min<int64_t>(buflen - 1, (int64_t)src.size());
        memcpy(buf, src.data(), (size_t)n);
        buf[n] = 0;
    }
    return (int64_t)src.size();
}

int gbh_validate(const gbh_batch_desc *desc, gbh_error *err, int64_t *n_neurons, int64_t *n_types)
{
    gbh_error local{};
    if (!err) err = &local;
    memset(err, 0, sizeof(*err));
    Decoded dec;
    int rc = decode_batch(desc, dec, err);
    if (rc) {
        set_last("%s", err->message);
        return rc;
    }
    std::map<std::string, int> keys;
    for (const Neuron &N : dec.neurons) keys[N.key] = 1;
    if (n_neurons) *n_neurons = (int64_t)dec.neurons.size();
    if (n_types) *n_types = (int64_t)keys.size();
    return GBH_OK;
}

gbh_engine *gbh_create(const gbh_batch_desc *desc, const gbh_synapses *syn, const gbh_options *opt,
                       gbh_error *err)
{
    return gbh_create_dist(desc, syn, nullptr, opt, err);
}

namespace {

gbh_engine *create_dist(const gbh_batch_desc *desc, const gbh_synapses *syn, const gbh_remote_synapses *remote,
                        const gbh_options *opt, gbh_error *err, gbh_engine *&made, const Decoded *pre = nullptr);

// The neuron-to-warp mapping, chosen by trial (gbh_options.wide_min 0): for
// each candidate -- neurons of at least 32, 64 or 128 compartments one per
// warp (wide tiles), or none (every large neuron lane-mapped, 32 per warp,
// with the stack elimination) -- an engine over the same decoded batch,
// interpreted (the specialised kernels serve the small types the same way
// under every candidate) at 16 steps per launch, times 32 steps after 16;
// the fastest candidate is kept. Returns the chosen wide_min.
// Also decides, when the kernel forms are autotuned (jit 0), whether the
// specialised kernels pay on this batch: they run beside the stack or wide
// launches and can slow the longest of them down (50,000 random trees: the
// 24 specialised kernels of the small neurons made the step 15-30 % slower).
// `no_jit` is set when the chosen mapping ran faster interpreted.
int choose_mapping(gbh_engine *e, const gbh_batch_desc *desc, const gbh_synapses *syn,
                   const gbh_remote_synapses *remote, bool &no_jit)
{
    no_jit = false;
    int maxrows = 0;
    for (const Neuron &N : e->dec.neurons) maxrows = std::max(maxrows, N.nrows);
    std::vector<int> cand;
    for (int w : {32, 64, 128})
        if (w <= maxrows) cand.push_back(w);
    if (cand.empty()) return -1;   // nothing large enough to run wide
    cand.push_back(-1);
    int best = cand[0];
    double best_ms = 1e300;
    // one trial: 32 steps after 16 on an engine built with the mapping w
    auto trial = [&](int w, int jit) {
        gbh_options o = e->opt;
        o.wide_min = w;
        o.jit = jit;
        o.steps_per_launch = 16;
        o.use_graph = 0;
        gbh_error te{};
        gbh_engine *made = nullptr, *t = nullptr;
        try {
            t = create_dist(desc, syn, remote, &o, &te, made, &e->dec);
        } catch (const std::exception &) {
            if (made) gbh_destroy(made);
            t = nullptr;
        }
        if (!t) return 1e300;   // a candidate that cannot be built is not chosen
        double ms = 1e300;
        if (gbh_run(t, 16) == GBH_OK) {
            const double ms0 = t->stats.device_ms;
            if (gbh_run(t, 32) == GBH_OK) ms = t->stats.device_ms - ms0;
        }
        if (getenv("GBH_VERBOSE"))
            fprintf(stderr, "gbhsolve: mapping trial wide_min %d%s: %.2f us/step (%lld wide, %lld stack tiles)\n", w,
                    jit < 0 ? "" : " specialised", ms / 32 * 1e3, (long long)t->stats.wide_tiles,
                    (long long)t->stats.stack_tiles);
        gbh_destroy(t);
        return ms;
    };
    for (int w : cand) {
        const double ms = trial(w, -1);
        if (ms < best_ms) {
            best_ms = ms;
            best = w;
        }
    }
    if (e->opt.jit == 0 && best_ms < 1e300) no_jit = trial(best, 0) > best_ms;
    return best;
}

gbh_engine *create_dist(const gbh_batch_desc *desc, const gbh_synapses *syn, const gbh_remote_synapses *remote,
                        const gbh_options *opt, gbh_error *err, gbh_engine *&made, const Decoded *pre)
{
    memset(err, 0, sizeof(*err));
    if (!desc) {
        fail_err(err, GBH_ERR_ARG, "NULL descriptor");
        return nullptr;
    }
    gbh_engine *e = new gbh_engine();
    made = e;
    if (opt) e->opt = *opt;
    e->nsolvers = desc->nsolvers;
    e->dt = desc->dt;
    if (cudaSetDevice(e->opt.device) != cudaSuccess) {
        fail_err(err, GBH_ERR_CUDA, "cudaSetDevice(%d) failed", e->opt.device);
        delete e;
        return nullptr;
    }
    int rc = GBH_OK;
    if (pre) e->dec = *pre;   // a trial engine over a batch already decoded
    else rc = decode_batch(desc, e->dec, err);
    if (rc) {
        set_last("%s", err->message);
        delete e;
        return nullptr;
    }
    if (!pre && e->opt.wide_min == 0) {
        bool no_jit = false;
        e->opt.wide_min = choose_mapping(e, desc, syn, remote, no_jit);
        if (no_jit) e->opt.jit = -1;
    }
    // keep the reference layout for state sync
    const int ns = desc->nsolvers;
    e->chip_start.assign(desc->chip_start, desc->chip_start + ns + 1);
    e->conc_start.assign(desc->conc_start, desc->conc_start + ns + 1);
    e->ops_start.assign(desc->ops_start, desc->ops_start + ns + 1);
    e->vm_start.assign(desc->vm_start, desc->vm_start + ns + 1);
    e->giv_start.assign(desc->givals_start, desc->givals_start + ns + 1);
    if (desc->storemode) e->itot_start.assign(desc->itotal_start, desc->itotal_start + ns + 1);
    else e->itot_start.assign(ns + 1, 0);
    e->rav_start.assign(desc->ravals_start, desc->ravals_start + ns + 1);
    e->chip_orig.assign(desc->chip, desc->chip + desc->chip_start[ns]);
    e->ops_orig.assign(desc->ops, desc->ops + desc->ops_start[ns]);
    rc = build_layout(e, desc, syn, remote, err);
    if (rc) {
        gbh_destroy(e);
        return nullptr;
    }
    if (e->launches.size() > 1) {
        const int ns = (int)std::min<size_t>(e->launches.size(), 8);
        e->side.resize(ns);
        e->ev_join.resize(ns);
        for (int i = 0; i < ns; ++i) {
            cudaStreamCreateWithFlags(&e->side[i], cudaStreamNonBlocking);
            cudaEventCreateWithFlags(&e->ev_join[i], cudaEventDisableTiming);
        }
        cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming);
    }
    if (e->d_step.alloc(1) || (e->has_network && e->d_gbar.upload(std::vector<unsigned>(3, 0u)))) {
        fail_err(err, GBH_ERR_CUDA, "%s", g_last_error);
        gbh_destroy(e);
        return nullptr;
    }
    e->steps_per_launch = e->opt.steps_per_launch > 0 ? e->opt.steps_per_launch : 64;
    bool wide_tiles = false;
    for (const TileType &tt : e->types) wide_tiles = wide_tiles || tt.wide;
    if (e->opt.steps_per_launch < 0 && e->has_network && e->nremote == 0 && !wide_tiles &&
        !e->spike_pre) {   // forced cooperative plan
        e->net_coop = true;
        e->net_spl = -e->opt.steps_per_launch;
    }
    if (e->has_network) e->steps_per_launch = 1;  // spikes cross tiles every step
    cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    cudaEventCreate(&e->ev0);
    cudaEventCreate(&e->ev1);
    if (e->opt.steps_per_launch == 0 && autotune(e) != GBH_OK) {
        fail_err(err, GBH_ERR_CUDA, "autotuner: %s", g_last_error);
        gbh_destroy(e);
        return nullptr;
    }
    int64_t comps = 0;
    for (const Neuron &N : e->dec.neurons) comps += N.nrows;
    e->stats.compartments = comps;
    e->stats.tiles = (int64_t)e->tiles.size();
    for (const Launch &L : e->launches) {
        if (L.wide) e->stats.wide_tiles += L.tile1 - L.tile0;
        if (L.stack) e->stats.stack_tiles += L.tile1 - L.tile0;
    }
    e->stats.precision = e->opt.precision;
    e->stats.steps_per_launch = e->net_coop ? e->net_spl : e->steps_per_launch;
    e->stats.cooperative = e->net_coop ? 1 : 0;
    e->stats.warps_per_block = e->launches.empty() ? 0 : e->launches[0].warps;
    if (!e->launches.empty() && e->launches[0].jit >= 0 && !e->jit_warps.empty())
        e->stats.warps_per_block = e->jit_warps[e->jit_choice];
    e->stats.jit_kernels = e->jit_compiled;
    e->stats.jit_min_blocks = e->jit_minb.empty() ? 0 : e->jit_minb[e->jit_choice];
    e->stats.jit_compact = e->jit_compact.empty() ? 0
                           : e->jit_compact[e->jit_choice] ? 1
                           : e->jit_smemrows[e->jit_choice] ? 2 : 0;
    if (getenv("GBH_VERBOSE"))
        for (const Launch &L : e->launches)
            fprintf(stderr, "gbhsolve: launch group tiles [%d, %d) smax %d %s\n", L.tile0, L.tile1, L.smax,
                    L.jit >= 0 ? "specialised" : "interpreted");
    if (getenv("GBH_VERBOSE") && !e->jit_log.empty())
        fprintf(stderr, "gbhsolve: specialised kernels: %d; compiler log:\n%.4000s\n", e->jit_compiled,
                e->jit_log.c_str());
    return e;
}

}  // namespace

// No C++ exception leaves the C ABI: running out of host memory (or threads)
// while building the engine is an error code, the partial engine released.
gbh_engine *gbh_create_dist(const gbh_batch_desc *desc, const gbh_synapses *syn, const gbh_remote_synapses *remote,
                            const gbh_options *opt, gbh_error *err)
{
    gbh_error local{};
    if (!err) err = &local;
    gbh_engine *made = nullptr;
    try {
        return create_dist(desc, syn, remote, opt, err, made);
    } catch (const std::exception &ex) {
        if (made) gbh_destroy(made);
        fail_err(err, GBH_ERR_ARG, "engine setup needs more host resources than are available (%s)", ex.what());
        return nullptr;
    }
}

int gbh_run_async(gbh_engine *e, int nsteps, void *stream)
{
    if (!e || nsteps < 0) return GBH_ERR_ARG;
    if (nsteps == 0) return GBH_OK;
    return run_steps(e, nsteps, stream ? (cudaStream_t)stream : e->stream);
}

int gbh_run(gbh_engine *e, int nsteps)
{
    if (!e || nsteps < 0) return GBH_ERR_ARG;
    if (nsteps == 0) return GBH_OK;
    CK(cudaEventRecord(e->ev0, e->stream));
    int rc = run_steps(e, nsteps, e->stream);
    if (rc) return rc;
    CK(cudaEventRecord(e->ev1, e->stream));
    CK(cudaEventSynchronize(e->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
    e->stats.device_ms += ms;
    e->stats.steps += nsteps;
    int status = 0;
    CK(cudaMemcpy(&status, e->d_status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (status) {
        set_last("device status word 0x%x (%s)", status,
                 (status & ST_SMEM)        ? "kernel launched with too little shared memory"
                 : (status & ST_NONFINITE) ? "a neuron's Vm is NaN or infinite"
                 : (status & ST_BARRIER)   ? "a grid barrier wait ran out"
                                           : "unimplemented micro-op reached");
        return GBH_ERR_DEVICE;
    }
    return GBH_OK;
}

int gbh_get_state(gbh_engine *e, double *vm, double *chip, double *conc, int *ops)
{
    if (!e) return GBH_ERR_ARG;
    const size_t L = LANES;
    CK(cudaStreamSynchronize(e->stream));
    std::vector<double> V(e->rows_vm * L), P(e->rows_fld * L), C(e->rows_pool * L);
    std::vector<int> I(e->rows_int * L);
    if (!V.empty()) CK(cudaMemcpy(V.data(), e->d_V.p, V.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (!P.empty()) CK(cudaMemcpy(P.data(), e->d_P.p, P.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (!C.empty()) CK(cudaMemcpy(C.data(), e->d_C.p, C.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (!I.empty()) CK(cudaMemcpy(I.data(), e->d_I.p, I.size() * sizeof(int), cudaMemcpyDeviceToHost));
    if (chip) memcpy(chip, e->chip_orig.data(), e->chip_orig.size() * sizeof(double));
    if (ops) memcpy(ops, e->ops_orig.data(), e->ops_orig.size() * sizeof(int));
    for (size_t i = 0; i < e->dec.neurons.size(); ++i) {
        const Neuron &N = e->dec.neurons[i];
        const Tile &t = e->tiles[e->neuron_tile[i]];
        const int l = e->neuron_lane[i];
        const bool w = e->types[t.type].wide != 0;
        if (vm)
            for (int s = 0; s < N.nrows; ++s) vm[e->vm_start[N.solver] + N.row0 + s] = V[at(t.vm, s, l, w)];
        const std::vector<char> &dfm = e->type_df[t.type];
        if (chip)
            for (size_t f = 0; f < N.fsrc.size(); ++f) {
                if (N.fsrc[f].kind != FS_CHIP) continue;
                const bool packed = !dfm.empty() && dfm[f];
                const double raw = P[at(t.fld, f, l, w)];
                // constants are reported as given; state and input-written
                // entries (the device copy changed) from the device
                if (!N.fsrc[f].state && raw == (packed ? pack_df(N.fval[f]) : N.fval[f])) continue;
                chip[e->chip_start[N.solver] + N.fsrc[f].idx] = packed ? unpack_df(raw) : raw;
            }
        if (conc)
            for (size_t p = 0; p < N.pool_conc.size(); ++p)
                conc[e->conc_start[N.solver] + N.pool_conc[p]] = C[at(t.pools, p, l, w)];
        if (ops)
            for (size_t r = 0; r < N.iops.size(); ++r)
                ops[e->ops_start[N.solver] + N.iops[r]] = I[at(t.ints, r, l, w)];
    }
    return GBH_OK;
}

int gbh_set_state(gbh_engine *e, const double *vm, const double *chip, const double *conc)
{
    if (!e) return GBH_ERR_ARG;
    const size_t L = LANES;
    CK(cudaStreamSynchronize(e->stream));
    std::vector<double> V(e->rows_vm * L), P(e->rows_fld * L), C(e->rows_pool * L);
    if (!V.empty()) CK(cudaMemcpy(V.data(), e->d_V.p, V.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (!P.empty()) CK(cudaMemcpy(P.data(), e->d_P.p, P.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (!C.empty()) CK(cudaMemcpy(C.data(), e->d_C.p, C.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < e->dec.neurons.size(); ++i) {
        const Neuron &N = e->dec.neurons[i];
        const Tile &t = e->tiles[e->neuron_tile[i]];
        const int l = e->neuron_lane[i];
        const bool w = e->types[t.type].wide != 0;
        if (vm)
            for (int s = 0; s < N.nrows; ++s) V[at(t.vm, s, l, w)] = vm[e->vm_start[N.solver] + N.row0 + s];
        const std::vector<char> &dfm = e->type_df[t.type];
        if (chip)
            for (size_t f = 0; f < N.fsrc.size(); ++f)
                if (N.fsrc[f].kind == FS_CHIP) {
                    const double val = chip[e->chip_start[N.solver] + N.fsrc[f].idx];
                    P[at(t.fld, f, l, w)] = (!dfm.empty() && dfm[f]) ? pack_df(val) : val;
                }
        if (conc)
            for (size_t p = 0; p < N.pool_conc.size(); ++p)
                C[at(t.pools, p, l, w)] = conc[e->conc_start[N.solver] + N.pool_conc[p]];
    }
    if (chip) e->chip_orig.assign(chip, chip + e->chip_orig.size());
    if (!V.empty()) CK(cudaMemcpy(e->d_V.p, V.data(), V.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (!P.empty()) CK(cudaMemcpy(e->d_P.p, P.data(), P.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (!C.empty()) CK(cudaMemcpy(e->d_C.p, C.data(), C.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (chip) {   // the stack tiles' kept factors come from chip fields
        const int rci = stack_invalidate(e, e->stream);
        if (rci) return rci;
        CK(cudaStreamSynchronize(e->stream));
    }
    return GBH_OK;
}

int gbh_enable_givals(gbh_engine *e, int enable)
{
    if (!e) return GBH_ERR_ARG;
    e->givals_enabled = enable != 0;
    e->givals_valid = false;
    return GBH_OK;
}

int gbh_get_givals(gbh_engine *e, double *givals)
{
    if (!e || !givals) return GBH_ERR_ARG;
    if (!e->givals_valid) {
        set_last("givals were not recorded: enable them before gbh_run");
        return GBH_ERR_ARG;
    }
    const size_t L = LANES;
    CK(cudaStreamSynchronize(e->stream));
    std::vector<double> Gv(e->rows_giv * L);
    if (!Gv.empty()) CK(cudaMemcpy(Gv.data(), e->d_giv.p, Gv.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < e->dec.neurons.size(); ++i) {
        const Neuron &N = e->dec.neurons[i];
        const Tile &t = e->tiles[e->neuron_tile[i]];
        const int l = e->neuron_lane[i];
        const bool w = e->types[t.type].wide != 0;
        for (size_t r = 0; r < N.giv_ref.size(); ++r)
            givals[e->giv_start[N.solver] + N.giv_ref[r]] = Gv[at(t.giv, r, l, w)];
    }
    return GBH_OK;
}

int gbh_get_itotal(gbh_engine *e, double *itotal)
{
    if (!e || !itotal) return GBH_ERR_ARG;
    if (e->rows_itot == 0) return GBH_OK;
    const size_t L = LANES;
    CK(cudaStreamSynchronize(e->stream));
    std::vector<double> It(e->rows_itot * L);
    CK(cudaMemcpy(It.data(), e->d_IT.p, It.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < e->dec.neurons.size(); ++i) {
        const Neuron &N = e->dec.neurons[i];
        const Tile &t = e->tiles[e->neuron_tile[i]];
        const int l = e->neuron_lane[i];
        for (int k = 0; k < N.nitot; ++k) itotal[e->itot_start[N.solver] + k] = It[at(t.itot, k, l, false)];
    }
    return GBH_OK;
}

int gbh_get_spiked(gbh_engine *e, uint8_t *solver_bits)
{
    if (!e || !solver_bits) return GBH_ERR_ARG;
    memset(solver_bits, 0, ((size_t)e->nsolvers + 7) / 8);
    if (!e->has_network) return GBH_OK;
    CK(cudaStreamSynchronize(e->stream));
    std::vector<unsigned> w(e->d_spiked.n);
    if (!w.empty()) CK(cudaMemcpy(w.data(), e->d_spiked.p, w.size() * sizeof(unsigned), cudaMemcpyDeviceToHost));
    CK(cudaMemsetAsync(e->d_spiked.p, 0, e->d_spiked.n * sizeof(unsigned), e->stream));
    for (size_t i = 0; i < e->dec.neurons.size(); ++i) {
        const Neuron &N = e->dec.neurons[i];
        if (N.spike_op < 0) continue;
        const int64_t g = e->tiles[e->neuron_tile[i]].first_neuron + e->neuron_lane[i];
        if (w[g >> 5] & (1u << (g & 31))) solver_bits[N.solver >> 3] |= (uint8_t)(1u << (N.solver & 7));
    }
    return GBH_OK;
}

int gbh_deliver_remote(gbh_engine *e, const uint8_t *source_bits)
{
    if (!e || !source_bits) return GBH_ERR_ARG;
    if (e->nremote == 0) return GBH_OK;
    if (e->step < 1) return fail_err(nullptr, GBH_ERR_ARG, "gbh_deliver_remote before the first step");
    const size_t nb = ((size_t)e->nremote + 7) / 8;
    CK(cudaMemcpyAsync(e->d_rbits.p, source_bits, nb, cudaMemcpyHostToDevice, e->stream));
    const int threads = 256, blocks = (e->nremote + threads - 1) / threads;
    k_deliver_remote<<<blocks, threads, 0, e->stream>>>(e->d_rbits.p, e->nremote, e->d_rstart.p, e->d_rbase.p,
                                                        e->d_rdelay.p, e->d_rmword.p, e->d_rmbit.p, e->d_ring.p,
                                                        e->d_wmask.p, e->ring_len, e->step - 1);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e->stream));   // the host bitmap may be reused on return
    e->stats.launches++;
    return GBH_OK;
}

int gbh_get_spike_counts(gbh_engine *e, int64_t *counts)
{
    if (!e || !counts) return GBH_ERR_ARG;
    CK(cudaStreamSynchronize(e->stream));
    std::vector<unsigned long long> s(e->d_spikes.n);
    if (!s.empty()) CK(cudaMemcpy(s.data(), e->d_spikes.p, s.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    for (int k = 0; k < e->nsolvers; ++k) counts[k] = 0;
    for (size_t i = 0; i < e->dec.neurons.size(); ++i) {
        const Neuron &N = e->dec.neurons[i];
        if (N.spike_op < 0) continue;
        const Tile &t = e->tiles[e->neuron_tile[i]];
        counts[N.solver] += (int64_t)s[t.first_neuron + e->neuron_lane[i]];
    }
    return GBH_OK;
}

int gbh_get_stats(const gbh_engine *e, gbh_stats *st)
{
    if (!e || !st) return GBH_ERR_ARG;
    *st = e->stats;
    return GBH_OK;
}

int gbh_loss_gradient(gbh_engine *e, int nsteps, int checkpoint_every, const gbh_loss_spec *spec,
                      double *loss, double *dchip, double *dravals, double *dvm0)
{
    if (!e || nsteps < 0 || !spec || spec->ntargets < 0 ||
        (spec->ntargets > 0 && (!spec->solver || !spec->row || !spec->trace)))
        return fail_err(nullptr, GBH_ERR_ARG, "gbh_loss_gradient: bad arguments");
    if (e->opt.precision != GBH_PREC_FP64)
        return fail_err(nullptr, GBH_ERR_UNSUPPORTED, "gbh_loss_gradient needs an FP64 engine");
    if (e->has_network)
        return fail_err(nullptr, GBH_ERR_UNSUPPORTED, "gbh_loss_gradient: synaptic networks are not differentiated");
    const size_t L = LANES;
    // ---- per type: supported program, plan tables ----
    std::vector<int> prog(e->d_prog.n);
    if (!prog.empty()) CK(cudaMemcpy(prog.data(), e->d_prog.p, prog.size() * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<AdjType> atypes(e->types.size());
    std::vector<int> snap_field;
    std::vector<AdjSlot> slot_plan;
    std::vector<AdjChan> chan_plan;
    for (size_t ti = 0; ti < e->types.size(); ++ti) {
        const TileType &tt = e->types[ti];
        if (tt.npools || tt.nsyn || tt.has_spike)
            return fail_err(nullptr, GBH_ERR_UNSUPPORTED,
                            "gbh_loss_gradient: Ca pools, synchans and spike detectors are not differentiated");
        if (tt.wide)
            return fail_err(nullptr, GBH_ERR_UNSUPPORTED,
                            "gbh_loss_gradient: create the engine with wide_min < 0 (one neuron per lane)");
        if (tt.sym)
            return fail_err(nullptr, GBH_ERR_UNSUPPORTED,
                            "gbh_loss_gradient: symmetric compartments are not differentiated");
        AdjType &at = atypes[ti];
        at.nslots = tt.nslots;
        at.snap_off = (int)snap_field.size();
        at.slot_off = (int)slot_plan.size();
        at.chan_off = (int)chan_plan.size();
        int pc = tt.prog_off, ek_field = -1, ngates = 0, nchans = 0;
        AdjSlot sp{};
        bool in_chan = false;
        for (int s = 0; s < tt.nslots;) {
            const int code = prog[pc];
            switch (code) {
            case M_BEGIN:
                sp = AdjSlot{};
                sp.f_emrm = prog[pc + 1];
                sp.f_inj = prog[pc + 2];
                sp.ch0 = nchans;
                pc += 5;
                break;
            case M_NEWVOLT:
                pc += 1;
                break;
            case M_CHAN:
            case M_CHAN_G: {
                if (in_chan)
                    return fail_err(nullptr, GBH_ERR_UNSUPPORTED, "gbh_loss_gradient: channel without ADD_CURR");
                AdjChan ch{};
                if (code == M_CHAN) ek_field = prog[pc + 1];
                ch.f_ek = ek_field;
                ch.f_gmax = prog[pc + (code == M_CHAN ? 2 : 1)];
                ch.g0 = ngates;
                chan_plan.push_back(ch);
                ++nchans;
                ++sp.nch;
                in_chan = true;
                pc += code == M_CHAN ? 3 : 2;
                break;
            }
            case M_GATE:
                if (!in_chan || prog[pc + 1] != GK_1V || prog[pc + 3] == 0)
                    return fail_err(nullptr, GBH_ERR_UNSUPPORTED,
                                    "gbh_loss_gradient: only voltage-table gates with a nonzero power are "
                                    "differentiated (kind %d, power %d)", prog[pc + 1], prog[pc + 3]);
                if (++chan_plan.back().ng > ADJ_MAX_GATES)
                    return fail_err(nullptr, GBH_ERR_UNSUPPORTED, "gbh_loss_gradient: more than %d gates in a channel",
                                    ADJ_MAX_GATES);
                snap_field.push_back(prog[pc + 4]);
                ++ngates;
                pc += 5;
                break;
            case M_ADDCURR:
                in_chan = false;
                pc += 2;
                break;
            case M_END:
                if (in_chan)
                    return fail_err(nullptr, GBH_ERR_UNSUPPORTED, "gbh_loss_gradient: channel without ADD_CURR");
                sp.f_tbyc = prog[pc + 1];
                sp.f_diag = prog[pc + 2];
                slot_plan.push_back(sp);
                pc += 4;
                ++s;
                break;
            default:
                return fail_err(nullptr, GBH_ERR_UNSUPPORTED,
                                "gbh_loss_gradient: micro-op %d (concentration, GHK, synaptic or pump terms) is "
                                "not differentiated", code);
            }
        }
        at.ngates = ngates;
        at.nchans = nchans;
        at.rows = adj_rows(tt.nslots, ngates, nchans).total;
    }
    if (nsteps == 0) {
        if (loss) *loss = 0.0;
        if (dchip) memset(dchip, 0, e->chip_start.back() * sizeof(double));
        if (dravals) memset(dravals, 0, e->rav_start.back() * sizeof(double));
        if (dvm0) memset(dvm0, 0, e->vm_start.back() * sizeof(double));
        return GBH_OK;
    }
    // K: the steps of one segment (tape); checkpoint_every <= 0 may keep every step instead
    const int K = std::max(1, std::min({checkpoint_every > 0 ? checkpoint_every : 100, nsteps, 65535}));
    const int nseg = (nsteps + K - 1) / K;
    // ---- target rows ----
    std::vector<int> tgt(e->rows_topo * L, -1);
    {
        std::unordered_map<int64_t, int> at;   // (solver, row) -> neuron
        for (size_t i = 0; i < e->dec.neurons.size(); ++i) {
            const Neuron &N = e->dec.neurons[i];
            for (int s = 0; s < N.nrows; ++s) at[(int64_t)N.solver * (1LL << 32) + N.row0 + s] = (int)i;
        }
        for (int j = 0; j < spec->ntargets; ++j) {
            auto it = at.find((int64_t)spec->solver[j] * (1LL << 32) + spec->row[j]);
            if (it == at.end())
                return fail_err(nullptr, GBH_ERR_ARG, "target %d: solver %d has no row %d", j, spec->solver[j],
                                spec->row[j]);
            const Neuron &N = e->dec.neurons[it->second];
            const Tile &t = e->tiles[e->neuron_tile[it->second]];
            int &cell = tgt[(t.topo + spec->row[j] - N.row0) * L + e->neuron_lane[it->second]];
            if (cell >= 0) return fail_err(nullptr, GBH_ERR_ARG, "target %d repeats target %d", j, cell);
            cell = j;
        }
    }
    // ---- checkpoint, tape and per-tile layouts ----
    const int ntiles = (int)e->tiles.size();
    std::vector<int64_t> ck_off(ntiles), tp_off(ntiles), xb_off(ntiles), ch_off(ntiles);
    int64_t ck_stride = 0, tp_stride = 0, xb_rows = 0, ch_rows = 0;
    int smax = 1, maxcopy = 1;
    for (int t = 0; t < ntiles; ++t) {
        const AdjType &at = atypes[e->tiles[t].type];
        ck_off[t] = ck_stride;
        tp_off[t] = tp_stride;
        xb_off[t] = xb_rows;
        ch_off[t] = ch_rows;
        ck_stride += at.nslots + at.ngates;
        tp_stride += at.rows;
        xb_rows += at.ngates;
        ch_rows += at.nchans;
        smax = std::max(smax, at.nslots);
        maxcopy = std::max(maxcopy, at.nslots + at.ngates);
    }
    if ((size_t)2 * smax * L * sizeof(double) > 200 * 1024)
        return fail_err(nullptr, GBH_ERR_UNSUPPORTED, "gbh_loss_gradient: %d compartments per neuron exceed shared memory",
                        smax);
    int hmax = 0;   // channel plans cached in shared memory by the reverse kernel
    for (const AdjType &at : atypes) hmax = std::max(hmax, at.nchans);
    while (hmax > 0 && adj_reverse_smem(smax, hmax) > 227 * 1024) hmax /= 2;
    // ---- device buffers (released on every return path) ----
    struct Bufs {
        DBuf<double> P, V, ck, tape, tape2, Vb, Xb, Gf, Gek, Ggm, GA, GB, GC, trace, loss;
        cudaStream_t ast = nullptr;
        cudaEvent_t ev_tape[2] = {nullptr, nullptr}, ev_done[2] = {nullptr, nullptr};
        DBuf<int> tgt, snap;
        DBuf<int64_t> ck_off, tp_off, xb_off, ch_off;
        DBuf<AdjType> atypes;
        DBuf<AdjSlot> slots;
        DBuf<AdjChan> chans;
        ~Bufs()
        {
            if (ast) cudaStreamSynchronize(ast);
            for (int i = 0; i < 2; ++i) {
                if (ev_tape[i]) cudaEventDestroy(ev_tape[i]);
                if (ev_done[i]) cudaEventDestroy(ev_done[i]);
            }
            if (ast) cudaStreamDestroy(ast);
            P.release(); V.release(); ck.release(); tape.release(); tape2.release(); Vb.release(); Xb.release();
            Gf.release();
            Gek.release(); Ggm.release(); GA.release(); GB.release(); GC.release(); trace.release();
            loss.release(); tgt.release(); snap.release(); ck_off.release(); tp_off.release(); xb_off.release();
            ch_off.release(); atypes.release(); slots.release(); chans.release();
        }
    } b;
    const int64_t nfld = e->rows_fld * L, nvm = e->rows_vm * L, ntopo = e->rows_topo * L;
    // checkpoint_every <= 0: every step's state kept (one checkpoint per
    // step) when it fits in 60% of the free memory beside the two tapes
    bool keep = false;
    if (checkpoint_every <= 0) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return fail_err(nullptr, GBH_ERR_CUDA, "cudaMemGetInfo");
        const double need = (double)nsteps * ck_stride * L * sizeof(double);
        const double tapes = 2.0 * K * tp_stride * L * sizeof(double);
        keep = need <= 0.6 * ((double)free_b - tapes);
        if (keep && b.ck.alloc((size_t)nsteps * ck_stride * L) != GBH_OK) {
            cudaGetLastError();
            keep = false;
        }
    }
    if ((!keep && b.ck.alloc((size_t)nseg * ck_stride * L)) || b.P.alloc(nfld) || b.V.alloc(nvm) ||
        b.tape.alloc((size_t)K * tp_stride * L) || b.Vb.alloc(nvm) || b.Xb.alloc(xb_rows * L) ||
        b.Gf.alloc(nfld) || b.Gek.alloc(ch_rows * L) || b.Ggm.alloc(ch_rows * L) || b.GA.alloc(ntopo) ||
        b.GB.alloc(ntopo) || b.GC.alloc(ntopo) || b.loss.alloc((size_t)ntiles * L) ||
        b.trace.alloc(std::max<size_t>(1, (size_t)nsteps * spec->ntargets)))
        return GBH_ERR_CUDA;
    if (b.tgt.upload(tgt) || b.snap.upload(snap_field) || b.ck_off.upload(ck_off) || b.tp_off.upload(tp_off) ||
        b.xb_off.upload(xb_off) || b.ch_off.upload(ch_off) || b.atypes.upload(atypes) ||
        b.slots.upload(slot_plan) || b.chans.upload(chan_plan))
        return GBH_ERR_CUDA;
    cudaStream_t st = e->stream;
    CK(cudaStreamSynchronize(st));
    if (spec->ntargets)
        CK(cudaMemcpy(b.trace.p, spec->trace, (size_t)nsteps * spec->ntargets * sizeof(double),
                      cudaMemcpyHostToDevice));
    CK(cudaMemcpyAsync(b.P.p, e->d_P.p, nfld * sizeof(double), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(b.V.p, e->d_V.p, nvm * sizeof(double), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemsetAsync(b.Vb.p, 0, nvm * sizeof(double), st));
    CK(cudaMemsetAsync(b.Xb.p, 0, std::max<int64_t>(1, xb_rows * L) * sizeof(double), st));
    CK(cudaMemsetAsync(b.Gf.p, 0, nfld * sizeof(double), st));
    CK(cudaMemsetAsync(b.Gek.p, 0, std::max<int64_t>(1, ch_rows * L) * sizeof(double), st));
    CK(cudaMemsetAsync(b.Ggm.p, 0, std::max<int64_t>(1, ch_rows * L) * sizeof(double), st));
    CK(cudaMemsetAsync(b.GA.p, 0, ntopo * sizeof(double), st));
    CK(cudaMemsetAsync(b.GB.p, 0, ntopo * sizeof(double), st));
    CK(cudaMemsetAsync(b.GC.p, 0, ntopo * sizeof(double), st));
    CK(cudaMemsetAsync(b.loss.p, 0, (size_t)ntiles * L * sizeof(double), st));
    AdjView v{};
    v.tiles = e->d_tiles.p;
    v.types = e->d_types.p;
    v.prog = e->d_prog.p;
    v.tgeom = e->d_tgeom.p;
    v.tab64 = e->d_tab64.p;
    v.xyvals = e->d_xy.p;
    v.parent = e->d_par.p;
    v.A = e->d_A.p;
    v.B = e->d_B.p;
    v.Cb = e->d_Cb.p;
    v.atypes = b.atypes.p;
    v.snap_field = b.snap.p;
    v.slot_plan = b.slots.p;
    v.chan_plan = b.chans.p;
    v.P = b.P.p;
    v.V = b.V.p;
    v.ckpt = b.ck.p;
    v.ck_off = b.ck_off.p;
    v.ck_stride = ck_stride;
    v.tape = b.tape.p;
    v.tp_off = b.tp_off.p;
    v.tp_stride = tp_stride;
    v.Vbar = b.Vb.p;
    v.Xbar = b.Xb.p;
    v.xb_off = b.xb_off.p;
    v.Gf = b.Gf.p;
    v.Gek = b.Gek.p;
    v.Ggm = b.Ggm.p;
    v.ch_off = b.ch_off.p;
    v.GA = b.GA.p;
    v.GB = b.GB.p;
    v.GC = b.GC.p;
    v.tgt = b.tgt.p;
    v.trace = b.trace.p;
    v.ntargets = spec->ntargets;
    v.loss = b.loss.p;
    v.status = e->d_status.p;
    // the engine's own FP64 step kernels advance the work copies
    DevView fv = view_of(e);
    fv.P = b.P.p;
    fv.V = b.V.p;
    auto ck_launch = [&](cudaError_t ce) {
        if (ce != cudaSuccess) {
            set_last("adjoint kernel launch failed: %s", cudaGetErrorString(ce));
            return GBH_ERR_CUDA;
        }
        return GBH_OK;
    };
    // the work copies' stack tiles keep their own factors (the engine's state
    // is restored afterwards; its tiles redo theirs at their next launch)
    if (stack_invalidate(e, st)) return GBH_ERR_CUDA;
    auto forward = [&](int n) { return issue_steps(e, fv, n, 0, false, st, nullptr); };
    // forward pass: checkpoints 0 .. nseg-1 (the last segment is recomputed),
    // or the state before every step when every step is kept
    CK(cudaEventRecord(e->ev0, st));
    if (keep) {
        for (int n = 0; n < nsteps; ++n) {
            if (ck_launch(launch_adj_copy(v, ntiles, maxcopy, n, 0, false, st))) return GBH_ERR_CUDA;
            if (n + 1 < nsteps && forward(1)) return GBH_ERR_CUDA;
        }
    } else {
        for (int seg = 0; seg < nseg; ++seg) {
            if (ck_launch(launch_adj_copy(v, ntiles, maxcopy, seg, 0, false, st))) return GBH_ERR_CUDA;
            if (seg + 1 < nseg && forward(K)) return GBH_ERR_CUDA;
        }
    }
    CK(cudaEventRecord(e->ev1, st));
    CK(cudaEventSynchronize(e->ev1));
    float ms_fwd = 0.f;
    CK(cudaEventElapsedTime(&ms_fwd, e->ev0, e->ev1));
    // reverse pass, segment by segment, last first: the snapshots into the
    // tape (recomputed from the checkpoint on the engine stream, or copied
    // when every step was kept), the linearisation, then sweep back and sum
    // the gradients (a second stream). With two tape buffers the next
    // segment's snapshots overlap this one's sweep; they share only the
    // constant fields of the work copy.
    const bool overlap = b.tape2.alloc((size_t)K * tp_stride * L) == GBH_OK;
    if (!overlap) cudaGetLastError();
    AdjView vb[2] = {v, v};
    if (overlap) vb[1].tape = b.tape2.p;
    CK(cudaStreamCreateWithFlags(&b.ast, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
        CK(cudaEventCreateWithFlags(&b.ev_tape[i], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&b.ev_done[i], cudaEventDisableTiming));
    }
    CK(cudaEventRecord(e->ev0, st));
    for (int idx = 0; idx < nseg; ++idx) {
        const int seg = nseg - 1 - idx;
        const int buf = overlap ? idx % 2 : 0;
        const AdjView &w = vb[buf];
        const int nk = std::min(K, nsteps - seg * K);
        // the buffer's previous segment must be through the adjoint kernels
        if (idx >= (overlap ? 2 : 1)) CK(cudaStreamWaitEvent(st, b.ev_done[buf], 0));
        if (keep) {
            if (ck_launch(launch_adj_ck_to_tape(w, ntiles, maxcopy, seg * K, nk, st))) return GBH_ERR_CUDA;
        } else {
            if (ck_launch(launch_adj_copy(w, ntiles, maxcopy, seg, 1, false, st))) return GBH_ERR_CUDA;
            for (int k = 0; k < nk; ++k) {
                if (ck_launch(launch_adj_copy(w, ntiles, maxcopy, k, 0, true, st))) return GBH_ERR_CUDA;
                if (k + 1 < nk && forward(1)) return GBH_ERR_CUDA;
            }
        }
        // the linearisation (parallel over steps): with every step kept, on
        // the engine stream, so that it overlaps the previous segment's
        // reverse sweep (a chain over steps on a few blocks); with segments
        // recomputed, beside the sweep on the second stream (the engine
        // stream runs the next segment's recomputation meanwhile)
        if (keep && ck_launch(launch_adj_linearize(w, ntiles, smax, nk, st))) return GBH_ERR_CUDA;
        CK(cudaEventRecord(b.ev_tape[buf], st));
        CK(cudaStreamWaitEvent(b.ast, b.ev_tape[buf], 0));
        if (!keep && ck_launch(launch_adj_linearize(w, ntiles, smax, nk, b.ast))) return GBH_ERR_CUDA;
        if (ck_launch(launch_adj_reverse(w, ntiles, smax, hmax, nk, seg * K, b.ast))) return GBH_ERR_CUDA;
        if (ck_launch(launch_adj_reduce(w, ntiles, smax, nk, b.ast))) return GBH_ERR_CUDA;
        CK(cudaEventRecord(b.ev_done[buf], b.ast));
    }
    CK(cudaEventRecord(b.ev_done[0], b.ast));
    CK(cudaStreamWaitEvent(st, b.ev_done[0], 0));
    CK(cudaEventRecord(e->ev1, st));
    CK(cudaEventSynchronize(e->ev1));
    float ms_rev = 0.f;
    CK(cudaEventElapsedTime(&ms_rev, e->ev0, e->ev1));
    e->stats.grad_forward_ms = ms_fwd;
    e->stats.grad_reverse_ms = ms_rev;
    e->stats.grad_kept_steps = keep ? 1 : 0;
    // forward step launches are counted by launch_one; add the copies
    // (checkpoint saves and restores, snapshots) and three kernels per segment
    e->stats.launches += (keep ? (int64_t)nsteps + nseg : 2 * (int64_t)nseg + nsteps) + 3 * (int64_t)nseg;
    int status = 0;
    CK(cudaMemcpy(&status, e->d_status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (status) {
        set_last("device status word 0x%x in the adjoint kernels", status);
        return GBH_ERR_DEVICE;
    }
    // ---- gather ----
    std::vector<double> Vb(nvm), Xb(xb_rows * L), Gf(nfld), Gek(ch_rows * L), Ggm(ch_rows * L), GA(ntopo),
        GB(ntopo), GC(ntopo), ls((size_t)ntiles * L);
    auto down = [&](std::vector<double> &h, const DBuf<double> &d) {
        if (h.empty()) return GBH_OK;
        CK(cudaMemcpy(h.data(), d.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
        return GBH_OK;
    };
    if (down(Vb, b.Vb) || down(Xb, b.Xb) || down(Gf, b.Gf) || down(Gek, b.Gek) || down(Ggm, b.Ggm) ||
        down(GA, b.GA) || down(GB, b.GB) || down(GC, b.GC) || down(ls, b.loss))
        return GBH_ERR_CUDA;
    if (loss) {
        double sum = 0.0;
        for (int t = 0; t < ntiles; ++t)
            for (int l = 0; l < e->tiles[t].nlanes; ++l) sum += ls[(size_t)t * L + l];
        *loss = sum;
    }
    if (dchip) memset(dchip, 0, e->chip_start.back() * sizeof(double));
    if (dravals) memset(dravals, 0, e->rav_start.back() * sizeof(double));
    if (dvm0) memset(dvm0, 0, e->vm_start.back() * sizeof(double));
    for (size_t i = 0; i < e->dec.neurons.size(); ++i) {
        const Neuron &N = e->dec.neurons[i];
        const int ti = e->neuron_tile[i];
        const Tile &t = e->tiles[ti];
        const AdjType &at = atypes[t.type];
        const int l = e->neuron_lane[i];
        if (dvm0)
            for (int s = 0; s < N.nrows; ++s) dvm0[e->vm_start[N.solver] + N.row0 + s] = Vb[(t.vm + s) * L + l];
        if (dchip) {
            // field gradients: per-slot fields, per-channel Ek and gmax, initial gate states
            std::vector<double> gfield(N.fsrc.size(), 0.0);
            for (size_t f = 0; f < N.fsrc.size(); ++f) gfield[f] = Gf[(t.fld + f) * L + l];
            for (int c = 0; c < at.nchans; ++c) {
                const AdjChan &ch = chan_plan[at.chan_off + c];
                if (ch.f_ek >= 0) gfield[ch.f_ek] += Gek[(ch_off[ti] + c) * L + l];
                gfield[ch.f_gmax] += Ggm[(ch_off[ti] + c) * L + l];
            }
            for (int g = 0; g < at.ngates; ++g) gfield[snap_field[at.snap_off + g]] += Xb[(xb_off[ti] + g) * L + l];
            for (size_t f = 0; f < N.fsrc.size(); ++f)
                if (N.fsrc[f].kind == FS_CHIP) dchip[e->chip_start[N.solver] + N.fsrc[f].idx] += gfield[f];
        }
        if (dravals)
            for (int s = 0; s < N.nrows; ++s) {
                const double g[3] = {GA[(t.topo + s) * L + l], GB[(t.topo + s) * L + l], GC[(t.topo + s) * L + l]};
                for (int q = 0; q < 3; ++q) {
                    const int r = N.ridx[3 * s + q];
                    if (r >= 0) dravals[e->rav_start[N.solver] + r] += g[q];
                }
            }
    }
    return GBH_OK;
}

void gbh_destroy(gbh_engine *e)
{
    if (!e) return;
    if (e->stream) cudaStreamSynchronize(e->stream);
    e->d_tiles.release(); e->d_types.release(); e->d_prog.release(); e->d_tgeom.release();
    e->d_tab64.release(); e->d_tab32.release(); e->d_tabdf.release(); e->d_xy.release(); e->d_P.release();
    e->d_V.release(); e->d_C.release(); e->d_F.release(); e->d_CR.release(); e->d_CD.release(); e->d_S.release(); e->d_wtop.release(); e->d_RV.release(); e->d_IT.release(); e->d_A.release(); e->d_B.release(); e->d_ltop.release(); e->d_col.release(); e->d_kst.release(); e->d_kri.release(); e->d_sgen.release(); e->d_tgen.release(); e->d_kref.release(); e->d_out_mword.release(); e->d_rmword.release(); e->d_out_mbit.release(); e->d_rmbit.release(); e->d_synw.release(); e->d_wval.release(); e->d_wmask.release(); e->d_spike_src.release();
    e->d_Cb.release(); e->d_giv.release(); e->d_stab.release(); e->d_I.release();
    e->d_par.release(); e->d_ring.release(); e->d_out_start.release(); e->d_out_base.release();
    e->d_out_delay.release(); e->d_spikes.release(); e->d_status.release();
    e->d_gbar.release(); e->d_spiked.release(); e->d_rstart.release(); e->d_rbase.release(); e->d_rdelay.release(); e->d_rbits.release();
    e->d_in_vals.release(); e->d_in_start.release(); e->d_in_addr.release();
    e->d_in_item.release(); e->d_in_sa.release(); e->d_in_sb.release();
    e->d_tin_start.release(); e->d_tin_off.release(); e->d_tin_idx.release();
    e->d_tout_start.release(); e->d_tout_off.release(); e->d_tout_idx.release();
    e->d_out_vals.release(); e->d_out_addr.release();
    drop_graphs(e);
    if (e->cap_stream) cudaStreamDestroy(e->cap_stream);
    for (cudaStream_t x : {e->io_stream, e->io_out_stream})
        if (x) {
            cudaStreamSynchronize(x);
            cudaStreamDestroy(x);
        }
    for (int b = 0; b < 2; ++b) {
        if (e->io_in_copied[b]) cudaEventDestroy(e->io_in_copied[b]);
        if (e->io_gathered[b]) cudaEventDestroy(e->io_gathered[b]);
        if (e->io_out_copied[b]) cudaEventDestroy(e->io_out_copied[b]);
        e->d_io_in[b].release();
        e->d_io_out[b].release();
        if (e->blk_in_copied[b]) cudaEventDestroy(e->blk_in_copied[b]);
        if (e->blk_done[b]) cudaEventDestroy(e->blk_done[b]);
        if (e->blk_out_copied[b]) cudaEventDestroy(e->blk_out_copied[b]);
        e->d_blk_in[b].release();
        e->d_blk_out[b].release();
    }
    for (cudaStream_t x : e->side) cudaStreamDestroy(x);
    for (cudaEvent_t x : e->ev_join) cudaEventDestroy(x);
    if (e->ev_fork) cudaEventDestroy(e->ev_fork);
    e->d_step.release();
    for (auto &vars : e->jit_var)
        for (JitKernel &k : vars) jit_release(k);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

}  // extern "C"
