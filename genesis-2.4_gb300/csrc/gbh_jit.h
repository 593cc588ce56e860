// gbh_jit.h -- per-program kernel specialisation (see gbh_jit.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gbh_devfn.cuh"

namespace gbh {

struct JitKernel {
    void *module = nullptr;   // CUmodule
    void *fn = nullptr;       // CUfunction
};

// CUDA source of the step kernel specialised to one tile type; empty if the
// program holds an op the generator does not emit. uniform_parent: the tree
// shared by every neuron of the type (elimination unrolled in registers), or
// null (per-neuron trees, shared-memory columns). compact: runs of identical
// compartment programs become loops and the rows stay in shared memory
// (smaller code; the autotuner decides which form runs). smem_rows: the
// unrolled form of a uniform tree keeps the eliminated rows (D, R) in
// shared-memory columns instead of registers, which frees ~4 registers a
// compartment for loads in flight.
std::string jit_source(const TileType &tt, const std::vector<int> &prog, const TableGeom &tg, bool mixed, bool giv,
                       const std::vector<int> *uniform_parent, int min_blocks = 4, bool compact = false,
                       bool smem_rows = false, int warps = 4);

bool jit_available(std::string *why);
int jit_compile(const std::string &src, bool fp64_exact, int device_major, int device_minor, JitKernel *out,
                std::string *log);
cudaError_t jit_launch(const JitKernel &k, const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                       long long step, size_t smem, cudaStream_t st);
void jit_release(JitKernel &k);

}  // namespace gbh
