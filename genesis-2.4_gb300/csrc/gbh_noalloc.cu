// gbh_noalloc.cu -- gbh_run_noalloc: advance an engine with no device
// allocation at all, for callers that may not allocate while stepping.
//
// The step kernel needs one per-step scratch area: the Ca flux rows that the
// channel programs accumulate (FLUX_OP / SCALE_FLUX_OP) and the pool update
// consumes. gbh_run takes it from the engine's own buffer; this entry point
// takes it from the fixed array below, which lives in the library image.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>

#include "gbhsolve.h"

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) double gbh_noalloc_flux[GBH_NOALLOC_FLUX_MAX];

int gbh_internal_run_with_flux(gbh_engine *e, int nsteps, cudaStream_t st, double *flux);
int64_t gbh_internal_flux_elems(const gbh_engine *e);
int gbh_internal_device(const gbh_engine *e);

namespace {
constexpr int kMaxDevices = 64;
double *g_flux_ptr[kMaxDevices] = {};
}  // namespace

extern "C" int gbh_run_noalloc(gbh_engine *e, int nsteps, void *stream)
{
    if (!e || nsteps < 0) return GBH_ERR_ARG;
    const int64_t need = gbh_internal_flux_elems(e);
    if (need > (int64_t)GBH_NOALLOC_FLUX_MAX) {
        fprintf(stderr,
                "gbh_run_noalloc: the engine needs %lld flux scratch doubles, the library's fixed "
                "buffer holds %d; use gbh_run\n",
                (long long)need, (int)GBH_NOALLOC_FLUX_MAX);
        return GBH_ERR_ARG;
    }
    const int dev = gbh_internal_device(e);
    if (dev < 0 || dev >= kMaxDevices) return GBH_ERR_ARG;
    if (cudaSetDevice(dev) != cudaSuccess) return GBH_ERR_CUDA;  // the engine's device is current
    if (!g_flux_ptr[dev]) {
        // once per device, with that device current: the host-side name of the
        // array is not a device address, so look the address up
        double *ptr = nullptr;
        if (cudaGetSymbolAddress((void **)&ptr, gbh_noalloc_flux) != cudaSuccess || !ptr) return GBH_ERR_CUDA;
        g_flux_ptr[dev] = ptr;
    }
    if (nsteps == 0) return GBH_OK;
    cudaStream_t st = (cudaStream_t)stream;
    // the array keeps the previous call's contents: start every call from zero
    if (need > 0 && cudaMemsetAsync(g_flux_ptr[dev], 0, (size_t)need * sizeof(double), st) != cudaSuccess)
        return GBH_ERR_CUDA;
    return gbh_internal_run_with_flux(e, nsteps, st, g_flux_ptr[dev]);
}
