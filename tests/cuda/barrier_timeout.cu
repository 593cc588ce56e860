// Test program: the engine's grid barrier (grid_sync, gbh_devfn.cuh) gives
// up after its poll limit when the arrivals it waits for never come, raises
// ST_BARRIER and returns, leaving the context usable. Two blocks wait for a
// third that is never launched -- a count that nothing completes, not a
// fault. Prints "status <word> gave_up <blocks> after <ms> ms context ok <0|1>".
#include <cstdio>

#include <cuda_runtime.h>

#include "gbh_devfn.cuh"

__global__ void k_wait(unsigned *bar, unsigned nblocks, int *status, int *gave_up)
{
    if (!gbh::grid_sync(bar, nblocks, status) && threadIdx.x == 0) atomicAdd(gave_up, 1);
}

__global__ void k_add(int *x) { atomicAdd(x, 1); }

int main()
{
    unsigned *bar = nullptr;
    int *word = nullptr;   // [0] status, [1] blocks that gave up, [2] a later kernel's count
    if (cudaMalloc(&bar, 3 * sizeof(unsigned)) != cudaSuccess || cudaMalloc(&word, 3 * sizeof(int)) != cudaSuccess)
        return 2;
    cudaMemset(bar, 0, 3 * sizeof(unsigned));
    cudaMemset(word, 0, 3 * sizeof(int));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0);
    k_wait<<<2, 32>>>(bar, 3u, word, word + 1);
    cudaEventRecord(e1);
    const cudaError_t ce = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    k_add<<<1, 32>>>(word + 2);
    const cudaError_t ce2 = cudaDeviceSynchronize();
    int h[3] = {0, 0, 0};
    cudaMemcpy(h, word, sizeof(h), cudaMemcpyDeviceToHost);
    printf("status %d gave_up %d after %.1f ms context ok %d\n", h[0], h[1], ms,
           (ce == cudaSuccess && ce2 == cudaSuccess && h[2] == 32) ? 1 : 0);
    return 0;
}
