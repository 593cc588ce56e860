// gbh_adjoint.h -- host/device interface of the adjoint kernels
// (gbh_adjoint.cuh, built in gbh_adjoint.cu) used by the engine's
// gbh_loss_gradient.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "gbh_internal.h"

namespace gbh {

constexpr int ADJ_MAX_GATES = 6;   // gates per channel the differentiated form handles

// Per tile type: counts and the offsets of its plan tables.
struct AdjType {
    int nslots, ngates, nchans;
    int rows;          // tape rows per step (see the row map below)
    int snap_off;      // into AdjView::snap_field: field row of every gate state, program order
    int slot_off;      // into AdjView::slot_plan: AdjSlot per slot
    int chan_off;      // into AdjView::chan_plan: AdjChan per channel, program order
};

// Field rows a slot's gradients go to, and its channels.
struct AdjSlot {
    int f_emrm, f_inj, f_tbyc, f_diag;
    int ch0, nch;      // channel ordinals [ch0, ch0 + nch)
};

struct AdjChan {
    int f_ek;          // field holding the Ek the channel uses (-1: none, Ek = 0)
    int f_gmax;
    int g0, ng;        // gate ordinals [g0, g0 + ng)
};

// Row map of one tile's block of one tape step (S slots, G gates, H channels):
//   V      [0, S)          Vm before the step          (snapshot)
//   ST     [S, S+G)        gate states before the step (snapshot)
//   RD     +S              1 / D' (final diagonal)
//   T      +S              A / D' (elimination factor, 0 at roots)
//   RP     +S              R' (final right-hand side)
//   X      +S              solution x
//   ICH    +S              ichan
//   SG     +S              sumg
//   PROD   +H              prod of x^p over the channel's gates
//   Q      +G              d prod / d x of each gate
//   DXDV   +G              d x' / d Vm of each gate (table slope, 0 if clamped)
//   DXDST  +G              d x' / d x (trapezoid factor, 0 for instant gates)
//   RBF    +S              adjoint of R (channel phase input)   (reverse)
//   DBF    +S              adjoint of D (channel phase input)   (reverse)
//   RBBS   +S              back-substitution adjoint r-bar      (reverse)
struct AdjRows {
    int V, ST, RD, T, RP, X, ICH, SG, PROD, Q, DXDV, DXDST, RBF, DBF, RBBS, total;
};

__host__ __device__ inline AdjRows adj_rows(int S, int G, int H)
{
    AdjRows r;
    r.V = 0;
    r.ST = S;
    r.RD = r.ST + G;
    r.T = r.RD + S;
    r.RP = r.T + S;
    r.X = r.RP + S;
    r.ICH = r.X + S;
    r.SG = r.ICH + S;
    r.PROD = r.SG + S;
    r.Q = r.PROD + H;
    r.DXDV = r.Q + G;
    r.DXDST = r.DXDV + G;
    r.RBF = r.DXDST + G;
    r.DBF = r.RBF + S;
    r.RBBS = r.DBF + S;
    r.total = r.RBBS + S;
    return r;
}

struct AdjView {
    const Tile *tiles;
    const TileType *types;
    const int *prog;
    const TableGeom *tgeom;
    const double *tab64;
    const double *xyvals;
    const int *parent;
    const double *A, *B, *Cb;
    const AdjType *atypes;
    const int *snap_field;
    const AdjSlot *slot_plan;
    const AdjChan *chan_plan;
    double *P;              // work fields (the forward passes advance the gate states)
    double *V;              // work vm
    double *ckpt;           // checkpoints: [c][tile block][lane], block = nslots + ngates rows
    const int64_t *ck_off;  // per tile: row offset of its block within one checkpoint
    int64_t ck_stride;      // rows per checkpoint
    double *tape;           // tape: [k][tile block][lane], block = AdjType::rows rows
    const int64_t *tp_off;  // per tile: row offset of its block within one tape step
    int64_t tp_stride;      // rows per tape step
    double *Vbar;           // vm rows: adjoint of Vm
    double *Xbar;           // per tile: ngates rows, adjoint of the gate states (gate ordinal)
    const int64_t *xb_off;  // per tile: row offset into Xbar
    double *Gf;             // field rows: gradients of Em/Rm, inject, tbyc, diagterm
    double *Gek, *Ggm;      // per tile: nchans rows, gradients of each channel's Ek and gmax
    const int64_t *ch_off;  // per tile: row offset into Gek / Ggm
    double *GA, *GB, *GC;   // topo rows: elimination-coefficient gradients
    const int *tgt;         // topo rows: trace column of the row or -1
    const double *trace;    // [step][ntargets]
    int ntargets;
    double *loss;           // per tile lane
    int *status;
};

// Checkpoint / snapshot copies between the work state and a block of
// nslots + ngates rows (Vm, then the gate states in program order); maxrows
// is the largest such block over the tile types.
//   dir 0: work -> checkpoint c, or -> tape step c when to_tape
//   dir 1: checkpoint c -> work
cudaError_t launch_adj_copy(const AdjView &v, int ntiles, int maxrows, int c, int dir, bool to_tape,
                            cudaStream_t st);
// Checkpoints c0 .. c0+nk-1 (one per step, every step's state kept) -> tape
// steps 0 .. nk-1.
cudaError_t launch_adj_ck_to_tape(const AdjView &v, int ntiles, int maxrows, int c0, int nk, cudaStream_t st);
// Per-step linearisation of tape steps [0, nk): recomputes each step from
// its snapshot (parallel over steps and tiles) and fills the tape rows.
cudaError_t launch_adj_linearize(const AdjView &v, int ntiles, int smax, int nk, cudaStream_t st);
// Reverse sweep over tape steps nk-1 .. 0 (step0: trace row of step 0);
// hmax: channels per neuron whose plan is cached in shared memory.
size_t adj_reverse_smem(int smax, int hmax);
cudaError_t launch_adj_reverse(const AdjView &v, int ntiles, int smax, int hmax, int nk, int step0, cudaStream_t st);
// Gradient sums of one segment's nk steps (parallel over tiles and slots).
cudaError_t launch_adj_reduce(const AdjView &v, int ntiles, int smax, int nk, cudaStream_t st);

}  // namespace gbh
