// Asynchronous work for sm_100+: mbarrier primitives with bounded waits, the bulk
// (TMA engine) global -> shared copy, and programmatic dependent launches (the
// device-side wait and trigger, and the host launcher that requests them).
#pragma once

#include <stdint.h>

#include <utility>

#include <cuda_runtime.h>

namespace gbfmm {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes the initialised barriers visible to the async proxy (bulk copies).
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Programmatic dependent launch (sm_90 and later).  A kernel launched with
// programmatic stream serialization (launch_k with pdl set) may start while the
// previous kernel of its stream is still running: it may stage constant tables
// first, but it calls pdl_wait() before it reads or writes anything that kernel
// touches.  pdl_wait returns once that kernel has completed and its writes are
// visible; in a plain launch it returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Lets the next kernel of the stream, if it was launched with programmatic
// serialization, start once every CTA of this grid has called this or exited.
// It only moves that kernel's start (its pdl_wait still waits for this grid's
// completion); without the call the next kernel starts when this grid ends.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Default poll limit of the bounded waits: 2^24 polls, well over a second.
constexpr uint32_t WAIT_POLLS_DEFAULT = 1u << 24;

// Bounded wait: gives up after 'limit' polls and ORs 'bit' into *err (when err
// is set).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int bit = 2,
                                          uint32_t limit = WAIT_POLLS_DEFAULT)
{
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicOr(err, bit);
    return false;
}

// Drain after a give-up: waits (again bounded, without reporting) for a phase
// whose asynchronous copies or MMAs were issued, so that a CTA does not release
// TMEM or exit while work it issued may still write its shared memory.
__device__ __forceinline__ bool mbar_drain(uint64_t* bar, uint32_t parity, uint32_t limit = WAIT_POLLS_DEFAULT)
{
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Bulk copy of 'bytes' (a multiple of 16; both addresses 16-byte aligned),
// completing on bar (tx bytes).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Launches kernel k on stream s; with pdl, as a programmatic dependent of the
// previous kernel of s (the kernel must call pdl_wait before it touches that
// kernel's data).  Captured into a graph, the dependency becomes a programmatic
// edge.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool pdl,
                            Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    if (pdl) {
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

}  // namespace gbfmm
