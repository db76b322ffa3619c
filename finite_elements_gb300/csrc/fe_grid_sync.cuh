// Grid-wide barrier with a bounded wait, for persistent kernels launched cooperatively
// (every block resident at once): the batched solver (fe_batch.cu) and the dense
// inverse of the multigrid's coarsest level (fe_amg_device_setup.cu).
//
// bar[0] counts the arrivals, bar[1] is the generation: thread 0 of each block reads
// the generation, arrives with an atomic, and the last to arrive resets the count and
// moves the generation on; the others poll it.  A poll that has not seen the
// generation move after kGridSpinLimit tries (about a second with the 64 ns sleeps)
// sets *err and stops waiting, and so does a block that sees *err already set: every
// block then returns false from its barrier and the kernel leaves, so a barrier never
// hangs the GPU.  bar and err start at zero.
#pragma once

namespace fe {
namespace {

constexpr unsigned kGridSpinLimit = 1u << 24;

__device__ __forceinline__ int ld_volatile_int(const int *p) { return *(const volatile int *)p; }

__device__ __forceinline__ bool grid_sync_bounded(unsigned *bar, int *err) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = bar + 1;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned spins = 0;
            while (*gen == g) {
                if (++spins > kGridSpinLimit || ld_volatile_int(err)) {
                    atomicExch(err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok = ld_volatile_int(err) == 0;
    }
    __syncthreads();
    return ok;
}

}  // namespace
}  // namespace fe
