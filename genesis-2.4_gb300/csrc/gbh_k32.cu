// gbh_k32.cu -- mixed-precision step kernels: gate and table arithmetic in
// double-float on FP32 instructions; Vm, elimination and Ca pools in FP64.
#include "gbh_kmixed.cuh"

namespace gbh {
cudaError_t launch_mixed(const DevView &v, int tile0, int tile1, int smax, int warps, int nsteps,
                         long long step, bool giv, cudaStream_t st)
{
    return launch_mixed_impl(v, tile0, tile1, smax, warps, nsteps, step, giv, st);
}

cudaError_t launch_mixed_wide(const DevView &v, int tile0, int tile1, int smax, int nsteps, long long step, bool giv,
                              cudaStream_t st)
{
    return giv ? wide_launch(k_wide_mixed<true>, v, tile0, tile1, smax, nsteps, step, st)
               : wide_launch(k_wide_mixed<false>, v, tile0, tile1, smax, nsteps, step, st);
}

cudaError_t launch_mixed_stack(const DevView &v, int tile0, int tile1, int cap, int nsteps, long long step,
                               bool giv, bool split, cudaStream_t st)
{
    return stack_launch_mixed(v, tile0, tile1, cap, nsteps, step, giv, split, st);
}

cudaError_t launch_mixed_coop(const DevView &v, int ntiles, int smax, int nsteps, long long step, cudaStream_t st)
{
    return coop_launch(k_steps_mixed<false>, v, ntiles, smax, nsteps, step, st);
}
}  // namespace gbh
