// gbh_adjoint.h -- host/device interface of the adjoint kernels
// (gbh_adjoint.cuh, built in gbh_adjoint.cu) used by the engine's
// gbh_loss_gradient.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "gbh_internal.h"

namespace gbh {

constexpr int ADJ_MAX_GATES = 6;   // gates per channel handled by the reverse step

struct AdjView {
    const Tile *tiles;
    const TileType *types;
    const int *prog;
    const TableGeom *tgeom;
    const double *tab64;
    const double *xyvals;
    const int *parent;
    const double *A, *B, *Cb;
    double *P;              // work fields (gate states advance)
    double *V;              // work vm
    double *ckpt;           // checkpoints: [c][tile block][lane], block = nslots + ngates rows
    const int64_t *ck_off;  // per tile: row offset of its block within one checkpoint
    int64_t ck_stride;      // rows per checkpoint
    double *tape;           // tape: [k][tile block][lane], block = 4*nslots + ngates rows
    const int64_t *tp_off;  // per tile: row offset of its block within one tape step
    int64_t tp_stride;      // rows per tape step
    double *Vbar;           // vm rows: adjoint of Vm
    double *Xbar;           // field rows: adjoint of gate states
    double *Gf;             // field rows: parameter gradients
    double *GA, *GB, *GC;   // topo rows: elimination-coefficient gradients
    const int *tgt;         // topo rows: trace column of the row or -1
    const double *trace;    // [step][ntargets]
    int ntargets;
    double *loss;           // per tile lane
    int *status;
};

cudaError_t launch_adj_forward(const AdjView &v, int tile0, int tile1, int smax, int nsteps, int K, int mode,
                               int seg, cudaStream_t st);
cudaError_t launch_adj_reverse(const AdjView &v, int tile0, int tile1, int smax, int nk, int step0,
                               cudaStream_t st);

}  // namespace gbh
