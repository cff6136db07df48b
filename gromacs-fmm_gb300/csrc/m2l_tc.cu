// Tensor-core M2L for sm_103a: tcgen05.mma (kind::f16, bf16 operands, FP32
// accumulation in TMEM) with split-precision operands.
//
// One CTA owns 128 targets of one (level, octant) stencil (M = 128 rows of the
// MMA = targets).  For each stencil entry e the CTA computes
//     D[t][:] += M~_src(t,e)[:] . T~_class(e)^T
// where the operator is split by output degree into "chunks": rows of degrees
// j0..j1 only see input degrees n <= P - j0 (the j+n<=P truncation of
// kernel.cu:585), so each chunk is an MMA of N = rows(j0..j1) (padded to 16) and
// K = (P-j0+1)^2 (padded to 16).  Operands are bf16 hi/lo splits of FP32 values;
// three products (hi*hi + hi*lo + lo*hi) keep ~16 bits (BF16X3), one product
// (hi*hi) ~8 bits (BF16X1).
//
// Data movement per entry and stage (two stages):
//   A (gathered source multipoles, 128 rows x K bf16, hi and lo): cp.async 16 B
//     copies into the canonical 128B-swizzled K-major layout;
//   B (operator chunk images, pre-swizzled on the host, hi and lo): one
//     cp.async.bulk (TMA engine) completing on an mbarrier.
// One thread issues the MMAs and commits them to the stage's "empty" mbarrier.
// Every wait is bounded; on timeout the kernel records an error and finishes.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>

#include "common.cuh"
#include "kernels.h"
#include "m2l_tc.h"

namespace gbfmm {

extern std::atomic<long> g_kernel_launches;

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

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

// Bounded wait: gives up after ~2^24 polls (well over a second) and flags the error.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err)
{
    for (uint32_t i = 0; i < (1u << 24); i++)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(err, 2);
    return false;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

// Arrives on the mbarrier once all of this thread's earlier cp.async copies have
// landed (the barrier's expected count includes this arrival).
__device__ __forceinline__ void cp_async_arrive_noinc(uint64_t* bar)
{
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Waits until at most n of this thread's most recent cp.async groups are pending.
__device__ __forceinline__ void cp_async_wait_pending(int n)
{
    switch (n) {
        case 0: asm volatile("cp.async.wait_group 0;" ::: "memory"); break;
        case 1: asm volatile("cp.async.wait_group 1;" ::: "memory"); break;
        case 2: asm volatile("cp.async.wait_group 2;" ::: "memory"); break;
        default: asm volatile("cp.async.wait_group 3;" ::: "memory"); break;
    }
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;           // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
    d |= (uint64_t)1 << 46;           // descriptor version
    d |= (uint64_t)2 << 61;           // 128-byte swizzle
    return d;
}

// Instruction descriptor: bf16 x bf16 -> f32, both K-major, M = 128, N.
__device__ __forceinline__ uint32_t idesc_bf16(int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace

// FP32 multipole rows -> bf16 hi/lo rows of TC_K elements (zero padded).
__global__ void k_split_bf16(const float* M, int Rpad, int R, long nrows, __nv_bfloat16* hi, __nv_bfloat16* lo)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    long row = i / TC_KMAX, c = i % TC_KMAX;
    if (row >= nrows) return;
    float x = c < R ? M[row * Rpad + c] : 0.f;
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    hi[row * TC_KMAX + c] = h;
    lo[row * TC_KMAX + c] = l;
}

void launch_split_bf16(const float* M, int Rpad, int R, long nrows, void* hi, void* lo, cudaStream_t s)
{
    long n = nrows * TC_KMAX;
    if (n <= 0) return;
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    k_split_bf16<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(M, Rpad, R, nrows, (__nv_bfloat16*)hi,
                                                               (__nv_bfloat16*)lo);
}

// Warp-specialised pipeline, no block-wide barrier in the main loop:
//   warps 0-3 (producers): thread t owns target row t; for entry i it waits until
//     stage i%NS is free (the MMAs of entry i-NS committed), gathers its source
//     row (cp.async, hi and lo bf16) into the 128B-swizzled A tile and arrives on
//     the stage's full barrier when its copies land (cp.async.mbarrier.arrive);
//     thread 0 also loads the operator images with one cp.async.bulk;
//   warp 4 (MMA issuer, one lane): waits for the full barrier, issues the chunked
//     tcgen05.mma sequence into TMEM and commits to the stage's empty barrier.
// After the last commit, warps 0-3 read their 32 TMEM lanes (tcgen05.ld) and add
// the results to the target locals.
__global__ void __launch_bounds__(TC_THREADS, 1) k_m2l_tc(TcArgs a)
{
    extern __shared__ uint8_t smraw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool split = a.nprod > 1;                    // lo halves are needed only for 3 products
    const int a_bytes = 128 * a.k_atoms * 128;        // one operand (hi or lo) of A
    const int b_bytes = a.img_bytes;                   // one operand of B
    const int stage_bytes = (split ? 2 : 1) * (a_bytes + b_bytes);
    const int NS = a.nstage;
    uint64_t* bar_full = reinterpret_cast<uint64_t*>(sm + NS * stage_bytes);
    uint64_t* bar_empty = bar_full + TC_MAXSTAGE;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_empty + TC_MAXSTAGE);

    const CTask task = a.tasks[blockIdx.x];
    if (tid == 0) {
        for (int k = 0; k < NS; k++) {
            mbar_init(&bar_full[k], 128 + 1);  // 128 producer copy arrivals + the bulk-copy expect_tx
            mbar_init(&bar_empty[k], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int ne = task.e_end - task.e_begin;
    bool ok = true;

    if (warp < 4) {
        // ---------------------------------------------------------------- producers
        const int t = tid;
        const bool tvalid = t < task.ntgt;
        int vt[3], va[3];
        const uint32_t q = (uint32_t)(task.q0 + t);
        const uint32_t tcode = (q << 3) | (uint32_t)task.octant;
        morton_decode(q, va[0], va[1], va[2]);
        morton_decode(tcode, vt[0], vt[1], vt[2]);
        const int chunks = a.k_atoms * 8;  // 16-byte chunks per row
        for (int i = 0; i < ne; i++) {
            const int st = i % NS, u = i / NS;
            if (i >= NS) ok = mbar_wait(&bar_empty[st], (u - 1) & 1, a.err) && ok;
            const CEntry en = a.entries[task.e_begin + i];
            uint8_t* A_hi = sm + st * stage_bytes;
            uint8_t* A_lo = A_hi + a_bytes;
            if (t == 0) {
                uint8_t* B = A_hi + (split ? 2 : 1) * a_bytes;
                const uint32_t nb = (split ? 2u : 1u) * b_bytes;
                mbar_expect_tx(&bar_full[st], nb);
                bulk_g2s(B, a.bimg + (size_t)en.op * 2 * b_bytes, nb, &bar_full[st]);
            }
            const int slev = en.mode == 0 ? task.level : task.level - 1;
            int row = -1;
            if (tvalid) {
                const int* base = en.mode == 0 ? vt : va;
                int sx = base[0] + en.dx, sy = base[1] + en.dy, sz = base[2] + en.dz;
                const int ns = 1 << slev;
                bool in = true;
                if (a.periodic) {
                    sx &= ns - 1; sy &= ns - 1; sz &= ns - 1;
                } else {
                    in = sx >= 0 && sy >= 0 && sz >= 0 && sx < ns && sy < ns && sz < ns;
                }
                if (in) row = (int)morton_encode(sx, sy, sz);
            }
            const bool valid = row >= 0;
            const size_t g0 = (size_t)(valid ? row : 0) * TC_KMAX;
            const __nv_bfloat16* gh = a.mh[slev] + g0;
            const __nv_bfloat16* gl = a.ml[slev] + g0;
            for (int kc = 0; kc < chunks; kc++) {
                const int soff = (kc >> 3) * (128 * 128) + t * 128 + (((kc & 7) ^ (t & 7)) << 4);
                cp_async16(A_hi + soff, gh + kc * 8, valid);
                if (split) cp_async16(A_lo + soff, gl + kc * 8, valid);
            }
            cp_async_arrive_noinc(&bar_full[st]);
        }
    } else if (lane == 0) {
        // ---------------------------------------------------------------- MMA issuer
        for (int i = 0; i < ne; i++) {
            const int st = i % NS, u = i / NS;
            ok = mbar_wait(&bar_full[st], u & 1, a.err) && ok;
            fence_proxy_async();
            tc_fence_after();
            const uint32_t a_hi = smem_u32(sm + st * stage_bytes), a_lo = a_hi + (uint32_t)a_bytes,
                           b_hi = a_hi + (uint32_t)((split ? 2 : 1) * a_bytes), b_lo = b_hi + (uint32_t)b_bytes;
            for (int c = 0; c < a.nchunk; c++) {
                const int N = a.chunk_n[c], K = a.chunk_k[c];
                const uint32_t idesc = idesc_bf16(N);
                const uint32_t boff = (uint32_t)a.chunk_img[c];
                for (int p = 0; p < a.nprod; p++) {
                    const uint32_t abase = p == 2 ? a_lo : a_hi;
                    const uint32_t bbase = (p == 1 ? b_lo : b_hi) + boff;
                    for (int kk = 0; kk < K / 16; kk++) {
                        const uint32_t ao = (uint32_t)((kk >> 2) * (128 * 128) + (kk & 3) * 32);
                        const uint32_t bo = (uint32_t)((kk >> 2) * (N * 128) + (kk & 3) * 32);
                        const uint32_t acc = (i > 0 || p > 0 || kk > 0) ? 1u : 0u;
                        mma_bf16(tmem + (uint32_t)a.chunk_col[c], sw128_desc(abase + ao), sw128_desc(bbase + bo),
                                 idesc, acc);
                    }
                }
            }
            mma_commit(&bar_empty[st]);
        }
    }
    // all MMAs complete (the last commit covers every earlier MMA of this thread)
    if (warp < 4 && ne > 0) ok = mbar_wait(&bar_empty[(ne - 1) % NS], ((ne - 1) / NS) & 1, a.err) && ok;
    __syncthreads();
    tc_fence_after();
    if (warp < 4 && ne > 0) {
        float* dst = a.dst_lvl[task.level];
        const int t = 32 * warp + lane;
        const bool wv = t < task.ntgt;
        const size_t trow = (size_t)(((uint32_t)(task.q0 + t) << 3) | (uint32_t)task.octant) * a.Rpad;
        for (int c = 0; c < a.nchunk; c++) {
            for (int b = 0; b < a.chunk_n[c]; b += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(a.chunk_col[c] + b), v);
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const int r = a.chunk_row0[c] + b + k;
                    if (wv && b + k < a.chunk_rows[c]) {
                        if (a.atomic) atomicAdd(&dst[trow + r], v[k]);
                        else dst[trow + r] += v[k];
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
    (void)ok;
}

size_t tc_stage_bytes(int k_atoms, int img_bytes, int nprod)
{
    return (size_t)(nprod > 1 ? 2 : 1) * ((size_t)128 * k_atoms * 128 + (size_t)img_bytes);
}

size_t tc_smem_bytes(const TcArgs& a)
{
    return 1024 + (size_t)a.nstage * tc_stage_bytes(a.k_atoms, a.img_bytes, a.nprod) +
           2 * TC_MAXSTAGE * sizeof(uint64_t) + 16;
}

// Stages per CTA: aim at two CTAs per SM (about 110 KB each), at least 2 stages.
int tc_pick_stages(int k_atoms, int img_bytes, int nprod)
{
    const size_t st = tc_stage_bytes(k_atoms, img_bytes, nprod);
    int ns = (int)((110 * 1024) / st);
    if (ns < 2) ns = 2;
    if (ns > TC_MAXSTAGE) ns = TC_MAXSTAGE;
    if (1024 + ns * st + 2 * TC_MAXSTAGE * sizeof(uint64_t) + 16 > 227 * 1024) ns = 1;
    return ns;
}

void launch_m2l_tc(const TcArgs& a, int ntasks, cudaStream_t s)
{
    if (ntasks <= 0) return;
    size_t shm = tc_smem_bytes(a);
    static size_t attr = 0;
    if (shm > attr) {
        cudaFuncSetAttribute(k_m2l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        attr = shm;
    }
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    k_m2l_tc<<<ntasks, TC_THREADS, shm, s>>>(a);
}

}  // namespace gbfmm
