// gbh_noalloc.cu -- gbh_run_noalloc: advance an engine with no device
// allocation at all, for callers that may not allocate while stepping.
//
// The step kernel needs one per-step scratch area: the Ca flux rows that the
// channel programs accumulate (FLUX_OP / SCALE_FLUX_OP), that FLUX messages
// set, and that the pool update consumes. gbh_run steps on the engine's own
// flux buffer; this entry point steps on the fixed array below, which lives
// in the library image. The engine's flux rows are copied into the array
// before the steps and back after them (device-to-device copies into memory
// that already exists), so FLUX inputs set with gbh_set_inputs_async and flux
// that a concentration carries from one step to the next are kept exactly as
// gbh_run keeps them.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>

#include "gbhsolve.h"

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) double gbh_noalloc_flux[GBH_NOALLOC_FLUX_MAX];

int gbh_internal_run_with_flux(gbh_engine *e, int nsteps, cudaStream_t st, double *flux);
int64_t gbh_internal_flux_elems(const gbh_engine *e);
double *gbh_internal_flux_rows(const gbh_engine *e);
int gbh_internal_device(const gbh_engine *e);
cudaStream_t gbh_internal_stream(const gbh_engine *e);

namespace {
constexpr int kMaxDevices = 64;
double *g_flux_ptr[kMaxDevices] = {};

int run_on_device(gbh_engine *e, int nsteps, void *stream, int dev, int64_t need)
{
    if (!g_flux_ptr[dev]) {
        // once per device, with that device current: the host-side name of the
        // array is not a device address, so look the address up
        double *ptr = nullptr;
        if (cudaGetSymbolAddress((void **)&ptr, gbh_noalloc_flux) != cudaSuccess || !ptr) return GBH_ERR_CUDA;
        g_flux_ptr[dev] = ptr;
    }
    if (nsteps == 0) return GBH_OK;
    // NULL means the engine's own stream, as for gbh_run_async
    cudaStream_t st = stream ? (cudaStream_t)stream : gbh_internal_stream(e);
    double *flux = g_flux_ptr[dev];
    const size_t bytes = (size_t)need * sizeof(double);
    // the array keeps the previous call's contents (another engine's, perhaps):
    // start from this engine's flux rows and hand them back afterwards
    if (need > 0 &&
        cudaMemcpyAsync(flux, gbh_internal_flux_rows(e), bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return GBH_ERR_CUDA;
    const int rc = gbh_internal_run_with_flux(e, nsteps, st, flux);
    if (rc) return rc;
    if (need > 0 &&
        cudaMemcpyAsync(gbh_internal_flux_rows(e), flux, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return GBH_ERR_CUDA;
    return GBH_OK;
}
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
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return GBH_ERR_CUDA;
    if (prev != dev && cudaSetDevice(dev) != cudaSuccess) return GBH_ERR_CUDA;  // the engine's device is current
    const int rc = run_on_device(e, nsteps, stream, dev, need);
    if (prev != dev) cudaSetDevice(prev);   // give the caller its device back
    return rc;
}
