// wave.cuh -- device helpers shared by the persistent wavefront kernels
// (SCFG inside/outside, posterior decoding): a grid barrier with a bounded
// wait and the split-sum group width.
#pragma once

#include "internal.h"

namespace messi {

// Largest CTA of the persistent wavefront kernels (their launch bounds).
constexpr int kWaveMaxThreads = 1024;

// ---------------------------------------------------------------------------
// grid barrier with a bounded wait (wavefront kernels)
// ---------------------------------------------------------------------------
// each spin is an L2 round trip plus a 32 ns sleep (~0.3-0.5 us): a wait gives
// up after one to two seconds
constexpr unsigned int kSpinLimit = 1u << 22;

static __device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Error bit of the arrival counter: a CTA that gives up waiting adds it, which
// ends every other CTA's wait (the count then exceeds any target) and tells it,
// from the same load, that the launch failed.
constexpr unsigned int kBarrierError = 1u << 30;

// sync[0] = arrivals, monotonic within a launch (barrier g completes when it
// reaches g * gridDim.x); sync[2] = error flag for the host.  Returns false
// (in every thread of the CTA) once any CTA has given up waiting.  Arrival is
// the cooperative-groups grid-barrier pattern: a CTA barrier, then thread 0's
// device-scope fence and atomic add; thread 0 polls with acquire loads and a
// second CTA barrier orders the other CTAs' cells before the CTA's next
// reads.  Cells written by other CTAs before the barrier are read with
// __ldcg (L2, coherent across SMs): the per-SM L1 may hold stale lines of
// those tables.  The barrier comes in two halves (grid_arrive, grid_wait) so
// that a CTA can work between its arrival and its wait on cells that do not
// depend on the other CTAs' latest writes; grid_sync is both at once.  Any
// thread may arrive for the CTA (`leader`): the fence waits for that
// thread's own loads still in flight, so a kernel that keeps loads in flight
// across its arrival picks a thread without any.
static __device__ __forceinline__ void grid_arrive(unsigned int* sync, unsigned int leader = 0)
{
    __syncthreads();
    if (threadIdx.x == leader) {
        __threadfence();
        atomicAdd(&sync[0], 1u);
    }
}

static __device__ bool grid_wait(unsigned int* sync, unsigned int& gen, unsigned int spin_limit = kSpinLimit)
{
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        const unsigned int target = (gen + 1) * gridDim.x;
        unsigned int v, spins = 0;
        while ((v = ld_acquire_u32(&sync[0])) < target) {
            if (++spins > spin_limit) {
                atomicExch(&sync[2], 1u);
                atomicAdd(&sync[0], kBarrierError);
                v = kBarrierError;
                break;
            }
            __nanosleep(32);
        }
        gen++;
        s_ok = (v & kBarrierError) == 0u;
    }
    __syncthreads();
    return s_ok != 0;
}

static __device__ bool grid_sync(unsigned int* sync, unsigned int& gen, unsigned int spin_limit = kSpinLimit)
{
    grid_arrive(sync);
    return grid_wait(sync, gen, spin_limit);
}

// Lanes per cell for a split sum of `nterms` terms: at most 8 terms per lane
// up to 256 terms, so a lane's loads are issued together and the sum costs
// one L2 round trip; longer sums use the whole warp.
static __device__ __forceinline__ int group_width(int nterms)
{
    return nterms <= 8 ? 1 : (nterms <= 16 ? 2 : (nterms <= 32 ? 4 : (nterms <= 64 ? 8 : (nterms <= 128 ? 16 : 32))));
}

}  // namespace messi
