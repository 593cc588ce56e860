// gbh_adjoint.cu -- launchers of the adjoint kernels (compiled with
// --fmad=false so the forward recomputation reproduces the FP64 step
// bit for bit).
#include "gbh_adjoint.cuh"

namespace gbh {

namespace {
cudaError_t smem_attr(const void *fn, size_t smem)
{
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
}  // namespace

cudaError_t launch_adj_forward(const AdjView &v, int tile0, int tile1, int smax, int nsteps, int K, int mode,
                               int seg, cudaStream_t st)
{
    const size_t smem = (size_t)2 * smax * LANES * sizeof(double);
    cudaError_t ce = smem_attr((const void *)k_adj_forward, smem);
    if (ce != cudaSuccess) return ce;
    k_adj_forward<<<tile1 - tile0, LANES, smem, st>>>(v, tile0, tile1, smax, nsteps, K, mode, seg);
    return cudaGetLastError();
}

cudaError_t launch_adj_reverse(const AdjView &v, int tile0, int tile1, int smax, int nk, int step0,
                               cudaStream_t st)
{
    const size_t smem = (size_t)2 * smax * LANES * sizeof(double);
    cudaError_t ce = smem_attr((const void *)k_adj_reverse, smem);
    if (ce != cudaSuccess) return ce;
    k_adj_reverse<<<tile1 - tile0, LANES, smem, st>>>(v, tile0, tile1, smax, nk, step0);
    return cudaGetLastError();
}

}  // namespace gbh
