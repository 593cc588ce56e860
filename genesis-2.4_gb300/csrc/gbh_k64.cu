// gbh_k64.cu -- FP64 step kernels (compiled with --fmad=false so the
// arithmetic matches the reference's CPU solver bit for bit).
#include "gbh_kernels.cuh"

namespace gbh {
cudaError_t launch_fp64(const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                        long long step, bool giv, cudaStream_t st)
{
    return launch_impl<double>(v, tile0, tile1, smax, warps, nsteps, step, giv, st);
}

cudaError_t launch_fp64_wide(const DevView &v, int tile0, int tile1, int smax, int nsteps, long long step, bool giv,
                             cudaStream_t st)
{
    return giv ? wide_launch(k_wide<double, true>, v, tile0, tile1, smax, nsteps, step, st)
               : wide_launch(k_wide<double, false>, v, tile0, tile1, smax, nsteps, step, st);
}

cudaError_t launch_fp64_stack(const DevView &v, int tile0, int tile1, int cap, int nsteps, long long step, bool giv,
                              bool split, cudaStream_t st)
{
    return stack_launch<double>(v, tile0, tile1, cap, nsteps, step, giv, split, st);
}

cudaError_t launch_fp64_coop(const DevView &v, int ntiles, int smax, int nsteps, long long step, cudaStream_t st)
{
    return coop_launch(k_steps<double, false>, v, ntiles, smax, nsteps, step, st);
}
}  // namespace gbh
