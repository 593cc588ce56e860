// gbh_adjoint.cu -- launchers of the adjoint kernels (compiled with
// --fmad=false so the per-step recomputation reproduces the FP64 step bit
// for bit).
#include "gbh_adjoint.cuh"

namespace gbh {

namespace {
cudaError_t smem_attr(const void *fn, size_t smem)
{
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
}  // namespace

cudaError_t launch_adj_copy(const AdjView &v, int ntiles, int maxrows, int c, int dir, bool to_tape,
                            cudaStream_t st)
{
    if (ntiles <= 0 || maxrows <= 0) return cudaSuccess;
    const dim3 grid(ntiles, (maxrows + 31) / 32);
    k_adj_copy<<<grid, LANES, 0, st>>>(v, c, dir, to_tape ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_adj_ck_to_tape(const AdjView &v, int ntiles, int maxrows, int c0, int nk, cudaStream_t st)
{
    if (ntiles <= 0 || maxrows <= 0 || nk <= 0) return cudaSuccess;
    const dim3 grid(ntiles, (maxrows + 31) / 32, nk);
    k_adj_ck_to_tape<<<grid, LANES, 0, st>>>(v, c0);
    return cudaGetLastError();
}

cudaError_t launch_adj_linearize(const AdjView &v, int ntiles, int smax, int nk, cudaStream_t st)
{
    if (ntiles <= 0 || nk <= 0) return cudaSuccess;
    const size_t smem = (size_t)2 * smax * LANES * sizeof(double);
    cudaError_t ce = smem_attr((const void *)k_adj_linearize, smem);
    if (ce != cudaSuccess) return ce;
    k_adj_linearize<<<dim3(ntiles, nk), LANES, smem, st>>>(v, smax);
    return cudaGetLastError();
}

size_t adj_reverse_smem(int smax, int hmax)
{
    return ((size_t)2 * smax * LANES + (size_t)ADJ_REV_WARPS * LANES) * sizeof(double) + (size_t)smax * sizeof(AdjSlot) +
           (size_t)hmax * sizeof(AdjChan);
}

cudaError_t launch_adj_reverse(const AdjView &v, int ntiles, int smax, int hmax, int nk, int step0, cudaStream_t st)
{
    if (ntiles <= 0 || nk <= 0) return cudaSuccess;
    const size_t smem = adj_reverse_smem(smax, hmax);
    cudaError_t ce = smem_attr((const void *)k_adj_reverse, smem);
    if (ce != cudaSuccess) return ce;
    k_adj_reverse<<<ntiles, ADJ_REV_WARPS * LANES, smem, st>>>(v, smax, hmax, nk, step0);
    return cudaGetLastError();
}

cudaError_t launch_adj_reduce(const AdjView &v, int ntiles, int smax, int nk, cudaStream_t st)
{
    if (ntiles <= 0 || nk <= 0) return cudaSuccess;
    k_adj_reduce<<<dim3(ntiles, smax), LANES, 0, st>>>(v, nk);
    return cudaGetLastError();
}

}  // namespace gbh
