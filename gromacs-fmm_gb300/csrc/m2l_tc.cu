// Tensor-core M2L for sm_103a: tcgen05.mma (kind::f16, bf16 operands, FP32
// accumulation in TMEM) with split-precision operands.
//
// One CTA owns a tile of up to 128 targets of one (level, octant): a box of
// bx x by x bz parent cells (M = 128 rows of the MMA, one per target).  For each
// stencil entry e of its range the CTA computes
//     D[t][:] += M~_src(t,e)[:] . T~_class(e)^T
// where the operator is split by output degree into "chunks": rows of degrees
// j0..j1 only see input degrees n <= P - j0 (the j+n<=P truncation of
// kernel.cu:585), so each chunk is an MMA of N = rows(j0..j1) (padded to 16) and
// K = (P-j0+1)^2 (padded to 16).  Operands are bf16 hi/lo splits of FP32 values;
// three products (hi*hi + hi*lo + lo*hi) keep ~16 bits (BF16X3), one product
// (hi*hi) ~8 bits (BF16X1).
//
// Data movement per entry and pipeline stage:
//   A (source multipoles of the tile): the sources of a tile for one entry are a
//     rectangular box of a halo-padded source grid (parity-split for same-level
//     sources, natural for parent-level sources), loaded by ONE TMA tile copy per
//     64-coefficient atom straight into the 128B-swizzled K-major layout;
//   B (operator chunk images, pre-swizzled on the host): one cp.async.bulk.
// One thread issues the copies, one thread the MMAs (committed to the stage's
// "empty" mbarrier); four warps read TMEM and add to the target locals.  Every
// wait is bounded; on timeout the kernel records an error and finishes.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>

#include "async.cuh"
#include "common.cuh"
#include "kernels.h"
#include "m2l_tc.h"

namespace gbfmm {

extern std::atomic<long> g_kernel_launches;

namespace {

// TMA tile loads of the source grids, completing on an mbarrier (tx bytes).
__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                            uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

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

// Target tile of level k: bx x by x bz parent cells (at most 8 x 4 x 4 = 128) of
// the stored parent grid (grid_n(k - 1, shift) cells per axis).
__host__ __device__ __forceinline__ void tc_tile_shape_dev(int level, const int* shift, int& bx, int& by, int& bz)
{
    const int mx = grid_n(level - 1, shift[0]), my = grid_n(level - 1, shift[1]), mz = grid_n(level - 1, shift[2]);
    bx = mx < 8 ? mx : 8;
    by = my < 4 ? my : 4;
    bz = mz < 4 ? mz : 4;
}

}  // namespace

// ------------------------------------------------------------------ source grids

// One thread per (grid row, 8 coefficients): the FP32 multipole of the row's
// cell (periodic image in the halo, zero outside a non-periodic box) split into
// bf16 hi and lo.
__device__ __forceinline__ void tc_grids_body(const TcGridArgs& g, const int bid)
{
    pdl_wait();
    pdl_trigger();
    const int groups = g.KP / 8;
    const long conv_blocks = ((g.rows - g.row_begin) * groups + 255) / 256;
    if (bid >= conv_blocks) {
        const int lane = threadIdx.x & 31, R = g.root_R;
        const int w = (int)(bid - conv_blocks) * 8 + (threadIdx.x >> 5);
        const int o = w / R, r = w % R;
        if (o >= g.root_n1) return;
        const double* A = g.root_l2l + ((size_t)o * R + r) * R;
        double t = 0;
        for (int c = lane; c < R; c += 32) t += A[c] * g.L0[c];
        for (int k = 16; k > 0; k >>= 1) t += __shfl_xor_sync(0xffffffffu, t, k);
        if (lane == 0) g.L1[(size_t)o * g.Rpad + r] += (float)t;
        return;
    }
    const long i = (long)bid * blockDim.x + threadIdx.x;
    if (i >= (g.rows - g.row_begin) * groups) return;
    const long row = g.row_begin + i / groups;
    const int c0 = (int)(i - (row - g.row_begin) * groups) * 8;
    int q = 0;
    while (q + 1 < g.ngrid && g.row0[q + 1] <= row) q++;
    long r = row - g.row0[q];
    const int Wx = g.W[q][0], Wy = g.W[q][1], Wz = g.W[q][2];
    const int nx = g.n[q][0], ny = g.n[q][1], nz = g.n[q][2];
    const int xh = (int)(r % Wx);
    r /= Wx;
    const int yh = (int)(r % Wy);
    r /= Wy;
    const int zh = (int)(r % Wz);
    r /= Wz;
    int x, y, z;
    if (g.parity[q]) {
        const int par = (int)r;
        x = 2 * (xh - TC_HALO) + (par & 1);
        y = 2 * (yh - TC_HALO) + ((par >> 1) & 1);
        z = 2 * (zh - TC_HALO) + (par >> 2);
    } else {
        x = xh - TC_HALO;
        y = yh - TC_HALO;
        z = zh - TC_HALO;
    }
    bool valid = true;
    if (g.periodic) {
        x = ((x % nx) + nx) % nx;
        y = ((y % ny) + ny) % ny;
        z = ((z % nz) + nz) % nz;
    } else {
        valid = x >= 0 && y >= 0 && z >= 0 && x < nx && y < ny && z < nz;
    }
    const float* src = g.src[q] + (size_t)(valid ? morton_encode(x, y, z) : 0u) * g.Rpad;
    alignas(16) __nv_bfloat16 h[8], l[8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
        const int c = c0 + e;
        const float v = valid && c < g.R ? src[c] : 0.f;
        h[e] = __float2bfloat16_rn(v);
        l[e] = __float2bfloat16_rn(v - __bfloat162float(h[e]));
    }
    *reinterpret_cast<uint4*>(g.hi + row * g.KP + c0) = *reinterpret_cast<const uint4*>(h);
    if (g.lo) *reinterpret_cast<uint4*>(g.lo + row * g.KP + c0) = *reinterpret_cast<const uint4*>(l);
}

__global__ void __launch_bounds__(256) k_tc_grids(const TcGridArgs g) { tc_grids_body(g, blockIdx.x); }

void launch_tc_grids(const TcGridArgs& g, cudaStream_t s, bool pdl)
{
    const long n = (g.rows - g.row_begin) * (g.KP / 8);
    if (n <= 0) return;
    const long root_blocks = g.root_l2l ? ((long)g.root_n1 * g.root_R + 7) / 8 : 0;
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    launch_k(k_tc_grids, dim3((unsigned)((n + 255) / 256 + root_blocks)), dim3(256), 0, s, pdl, g);
}

// ------------------------------------------------------------------ M2L

// Warp-specialised pipeline, no block-wide barrier in the main loop:
//   warp 0, lane 0 (producer): for entry i it waits until stage i%NS is free (the
//     MMAs of entry i-NS committed), then issues the TMA tile loads of the source
//     box (one per K atom, hi and lo) and the bulk copy of the operator images,
//     all completing on the stage's full barrier;
//   warp 1, lane 0 (MMA issuer): waits for the full barrier, issues the chunked
//     tcgen05.mma sequence into TMEM and commits to the stage's empty barrier.
// After the last commit, warps 0-3 read their 32 TMEM lanes (tcgen05.ld) and add
// the results to the target locals.
__device__ __forceinline__ void m2l_tc_body(const TcArgs& a, const int bid)
{
    extern __shared__ uint8_t smraw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool split = a.nprod > 1;                    // lo halves are needed only for 3 products
    const int a_bytes = 128 * a.k_atoms * 128;        // one operand (hi or lo) of A
    const int b_bytes = a.img_bytes;                   // one operand of B
    const int slot_bytes = (split ? 2 : 1) * (a_bytes + b_bytes);  // the operands of one entry
    const int G = a.group;                             // entries per pipeline stage
    const int stage_bytes = G * slot_bytes;
    const int NS = a.nstage;
    uint64_t* bar_full = reinterpret_cast<uint64_t*>(sm + NS * stage_bytes);
    uint64_t* bar_empty = bar_full + TC_MAXSTAGE;
    uint64_t* bar_done = bar_empty + TC_MAXSTAGE;  // one phase: every MMA of the CTA has completed
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_done + 1);

    const CTask task = a.tasks[bid];
    const int k = task.level, s = task.octant;
    int bx, by, bz;
    tc_tile_shape_dev(k, a.shift, bx, by, bz);
    const int tx = grid_n(k - 1, a.shift[0]) / bx, ty = grid_n(k - 1, a.shift[1]) / by;
    const int i0 = (task.q0 % tx) * bx, j0 = ((task.q0 / tx) % ty) * by, l0 = (task.q0 / (tx * ty)) * bz;
    const int rows = bx * by * bz;
    const int ox = (s >> 2) & 1, oy = (s >> 1) & 1, oz = s & 1;

    // the task's stencil entries, read once (the producer must not wait on
    // global loads between its copies); their loads overlap the vacuum test's
    __shared__ CEntry ent[TC_MAXENT];
    const int ne = min(task.e_end - task.e_begin, TC_MAXENT);
    for (int i = tid; i < ne; i += TC_THREADS) ent[i] = a.entries[task.e_begin + i];

    // a tile whose targets hold no bodies (vacuum) needs no locals: their only
    // readers are their own descendants' L2P
    if (a.leaf_off) {
        bool occupied = false;
        if (tid < rows) {
            const int bi = tid % bx, bj = (tid / bx) % by, bl = tid / (bx * by);
            const uint32_t code = (morton_encode(i0 + bi, j0 + bj, l0 + bl) << 3) | (uint32_t)s;
            const int sh = 3 * (a.depth - k);
            occupied = a.leaf_off[(code + 1) << sh] > a.leaf_off[code << sh];
        }
        if (!__syncthreads_or(occupied)) return;
    }

    if (tid == 0) {
        for (int q = 0; q < NS; q++) {
            mbar_init(&bar_full[q], 1);
            mbar_init(&bar_empty[q], 1);
        }
        mbar_init(bar_done, 1);
        mbar_init_fence();
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lim = a.wait_limit;
    bool ok = true;
    // the set-up above reads only this step's tree and constant lists; the source
    // grids and the locals belong to the previous kernel (a programmatic launch)
    pdl_wait();

    // On a bounded wait that gives up, the waiting role records the error, stops
    // issuing work and drains what it issued (again bounded); the CTA then skips
    // the read-back and the adds, and releases TMEM only after the drain.
    const int ng = (ne + G - 1) / G;  // stage uses: groups of G entries
    if (warp == 0 && lane == 0) {
        // ---------------------------------------------------------------- producer
        const uint32_t tx_entry = (split ? 2u : 1u) * (uint32_t)(a.k_atoms * rows * 128 + b_bytes);
        int issued = 0;
        for (int g = 0; g < ng; g++) {
            const int st = g % NS, u = g / NS;
            if (g >= NS && !mbar_wait(&bar_empty[st], (u - 1) & 1, a.err, 2, lim)) {
                ok = false;
                break;
            }
            const int e0 = g * G, e1 = min(ne, e0 + G);
            mbar_expect_tx(&bar_full[st], (uint32_t)(e1 - e0) * tx_entry);
            for (int i = e0; i < e1; i++) {
                const CEntry en = ent[i];
                uint8_t* A_hi = sm + st * stage_bytes + (i - e0) * slot_bytes;
                uint8_t* A_lo = A_hi + a_bytes;
                uint8_t* B = A_hi + (split ? 2 : 1) * a_bytes;
                if (en.mode == 0) {
                    // same-level source: parity grid of level k
                    const int fx = (ox + en.dx) >> 1, fy = (oy + en.dy) >> 1, fz = (oz + en.dz) >> 1;
                    const int par = ((ox + en.dx) & 1) | (((oy + en.dy) & 1) << 1) | (((oz + en.dz) & 1) << 2);
                    const int cx = i0 + fx + TC_HALO, cy = j0 + fy + TC_HALO, cz = l0 + fz + TC_HALO;
                    for (int at = 0; at < a.k_atoms; at++) {
                        tma_load_5d(A_hi + at * 128 * 128, &a.p_hi[k], 64 * at, cx, cy, cz, par, &bar_full[st]);
                        if (split) tma_load_5d(A_lo + at * 128 * 128, &a.p_lo[k], 64 * at, cx, cy, cz, par, &bar_full[st]);
                    }
                } else {
                    // parent-level source: natural grid of level k-1
                    const int cx = i0 + en.dx + TC_HALO, cy = j0 + en.dy + TC_HALO, cz = l0 + en.dz + TC_HALO;
                    for (int at = 0; at < a.k_atoms; at++) {
                        tma_load_4d(A_hi + at * 128 * 128, &a.n_hi[k - 1], 64 * at, cx, cy, cz, &bar_full[st]);
                        if (split) tma_load_4d(A_lo + at * 128 * 128, &a.n_lo[k - 1], 64 * at, cx, cy, cz, &bar_full[st]);
                    }
                }
                bulk_g2s(B, a.bimg + (size_t)en.op * 2 * b_bytes, (split ? 2u : 1u) * b_bytes, &bar_full[st]);
            }
            issued = g + 1;
        }
        if (!ok)  // the copies this thread issued: the last phase of every stage
            for (int st = 0; st < min(NS, issued); st++) mbar_drain(&bar_full[st], ((issued - 1 - st) / NS) & 1, lim);
    } else if (warp == 1 && lane == 0) {
        // ---------------------------------------------------------------- MMA issuer
        for (int g = 0; g < ng; g++) {
            const int st = g % NS, u = g / NS;
            if (!mbar_wait(&bar_full[st], u & 1, a.err, 2, lim)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const int e0 = g * G, e1 = min(ne, e0 + G);
            for (int i = e0; i < e1; i++) {
                const uint32_t a_hi = smem_u32(sm + st * stage_bytes + (i - e0) * slot_bytes),
                               a_lo = a_hi + (uint32_t)a_bytes, b_hi = a_hi + (uint32_t)((split ? 2 : 1) * a_bytes),
                               b_lo = b_hi + (uint32_t)b_bytes;
                // descriptors of the entry's operands; an offset of o bytes (a multiple
                // of 16, within the 256 KB shared window) adds o >> 4 to the start field
                const uint64_t da_hi = sw128_desc(a_hi), da_lo = sw128_desc(a_lo), db_hi = sw128_desc(b_hi),
                               db_lo = sw128_desc(b_lo);
                for (int c = 0; c < a.nchunk; c++) {
                    const int N = a.chunk_n[c], K = a.chunk_k[c];
                    const uint32_t idesc = idesc_bf16(N);
                    const uint32_t dcol = tmem + (uint32_t)a.chunk_col[c];
                    const uint64_t boff = (uint64_t)(a.chunk_img[c] >> 4);
                    for (int p = 0; p < a.nprod; p++) {
                        const uint64_t da = p == 2 ? da_lo : da_hi;
                        const uint64_t db = (p == 1 ? db_lo : db_hi) + boff;
                        for (int kk = 0; kk < K / 16; kk++) {
                            const uint64_t ao = (uint64_t)((kk >> 2) * (128 * 128 / 16) + (kk & 3) * 2);
                            const uint64_t bo = (uint64_t)((kk >> 2) * (N * 128 / 16) + (kk & 3) * 2);
                            const uint32_t acc = (i > 0 || p > 0 || kk > 0) ? 1u : 0u;
                            mma_bf16(dcol, da + ao, db + bo, idesc, acc);
                        }
                    }
                }
            }
            mma_commit(&bar_empty[st]);
        }
        // completes when every MMA issued above has completed; only this thread
        // polls it (a parity wait on a stage barrier could pass before that
        // barrier's first phase completes), the others wait at the CTA barrier
        if (ne > 0) {
            mma_commit(bar_done);
            if (!mbar_wait(bar_done, 0, a.err, 2, lim)) {
                ok = false;
                mbar_drain(bar_done, 0, lim);
            }
        }
    }
    tc_fence_before();
    const bool failed = __syncthreads_or(!ok) != 0;
    tc_fence_after();
    pdl_trigger();  // only the epilogue is left: the next kernel may launch (it waits for this one's end)
    if (ne > 0 && !failed) {
        float* dst = a.dst_lvl[k];
        const int t = 32 * warp + lane;
        const bool wv = t < rows;
        const int bi = t % bx, bj = (t / bx) % by, bl = t / (bx * by);
        const uint32_t q = wv ? morton_encode(i0 + bi, j0 + bj, l0 + bl) : 0u;
        const size_t trow = (size_t)((q << 3) | (uint32_t)s) * a.Rpad;
        for (int c = 0; c < a.nchunk; c++) {
            // rows r0 + b .. in groups of 4: one vector add (or atomic vector add) where
            // the group is whole and 16-byte aligned (Rpad is a multiple of 4)
            const bool al = (a.chunk_row0[c] & 3) == 0;
            for (int b = 0; b < a.chunk_n[c]; b += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(a.chunk_col[c] + b), v);
                if (!wv) continue;
#pragma unroll
                for (int e = 0; e < 16; e += 4) {
                    const int r = a.chunk_row0[c] + b + e;
                    float* d = &dst[trow + r];
                    if (al && b + e + 3 < a.chunk_rows[c]) {
                        if (a.atomic) {
                            asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(d), "f"(v[e]),
                                         "f"(v[e + 1]), "f"(v[e + 2]), "f"(v[e + 3])
                                         : "memory");
                        } else {
                            float4 t = *reinterpret_cast<float4*>(d);
                            t.x += v[e];
                            t.y += v[e + 1];
                            t.z += v[e + 2];
                            t.w += v[e + 3];
                            *reinterpret_cast<float4*>(d) = t;
                        }
                    } else {
#pragma unroll
                        for (int f = 0; f < 4; f++) {
                            if (b + e + f < a.chunk_rows[c]) {
                                if (a.atomic) atomicAdd(d + f, v[e + f]);
                                else d[f] += v[e + f];
                            }
                        }
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 2)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
    (void)ok;
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_m2l_tc(const __grid_constant__ TcArgs a) { m2l_tc_body(a, blockIdx.x); }

// ------------------------------------------------------------------ host side

void tc_tile_shape(int level, const int shift[3], int& bx, int& by, int& bz)
{
    tc_tile_shape_dev(level, shift, bx, by, bz);
}

int tc_tiles(int level, const int shift[3])
{
    int bx, by, bz;
    tc_tile_shape(level, shift, bx, by, bz);
    return (grid_n(level - 1, shift[0]) / bx) * (grid_n(level - 1, shift[1]) / by) *
           (grid_n(level - 1, shift[2]) / bz);
}

bool tc_octant_stored(int level, const int shift[3], int octant)
{
    for (int d = 0; d < 3; d++)
        if (grid_n(level, shift[d]) == 1 && ((octant >> (2 - d)) & 1)) return false;
    return true;
}

TcGrids tc_grid_layout(int D, int k_atoms, const int shift[3])
{
    TcGrids g;
    g.KP = 64 * k_atoms;
    long rows = 0;
    for (int k = 0; k <= D; k++) {
        if (k < D) {  // natural grid: parent-level sources of level k+1
            for (int d = 0; d < 3; d++) g.n_w[k][d] = grid_n(k, shift[d]) + 2 * TC_HALO;
            g.n_row0[k] = rows;
            rows += (long)g.n_w[k][0] * g.n_w[k][1] * g.n_w[k][2];
        }
        if (k >= 1) {  // parity grid: same-level sources of level k
            for (int d = 0; d < 3; d++) g.p_w[k][d] = (grid_n(k, shift[d]) + 1) / 2 + 2 * TC_HALO;
            g.p_row0[k] = rows;
            rows += 8L * g.p_w[k][0] * g.p_w[k][1] * g.p_w[k][2];
        }
    }
    g.rows = rows;
    return g;
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// rank-4 (natural) or rank-5 (parity) map of one grid: dims (KP, Wx, Wy, Wz[, 8]),
// box (64, bx, by, bz[, 1]) of the target level's tile, 128-byte swizzle
static bool encode_grid(CUtensorMap* map, void* base, int KP, const int* W, bool parity, int bx, int by, int bz)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint32_t rank = parity ? 5 : 4;
    cuuint64_t dims[5] = {(cuuint64_t)KP, (cuuint64_t)W[0], (cuuint64_t)W[1], (cuuint64_t)W[2], 8};
    const cuuint64_t row = (cuuint64_t)KP * 2;
    cuuint64_t strides[4] = {row, row * W[0], row * W[0] * W[1], row * W[0] * W[1] * W[2]};
    cuuint32_t box[5] = {64, (cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz, 1};
    cuuint32_t es[5] = {1, 1, 1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, rank, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool tc_encode_maps(TcArgs& a, int D, const TcGrids& g, void* hi, void* lo)
{
    __nv_bfloat16* h = static_cast<__nv_bfloat16*>(hi);
    __nv_bfloat16* l = static_cast<__nv_bfloat16*>(lo);
    for (int k = 1; k <= D; k++) {
        int bx, by, bz;
        tc_tile_shape(k, a.shift, bx, by, bz);
        if (!encode_grid(&a.p_hi[k], h + g.p_row0[k] * g.KP, g.KP, g.p_w[k], true, bx, by, bz)) return false;
        if (!encode_grid(&a.n_hi[k - 1], h + g.n_row0[k - 1] * g.KP, g.KP, g.n_w[k - 1], false, bx, by, bz))
            return false;
        if (l) {
            if (!encode_grid(&a.p_lo[k], l + g.p_row0[k] * g.KP, g.KP, g.p_w[k], true, bx, by, bz)) return false;
            if (!encode_grid(&a.n_lo[k - 1], l + g.n_row0[k - 1] * g.KP, g.KP, g.n_w[k - 1], false, bx, by, bz))
                return false;
        }
    }
    return true;
}

size_t tc_stage_bytes(int k_atoms, int img_bytes, int nprod)
{
    return (size_t)(nprod > 1 ? 2 : 1) * ((size_t)128 * k_atoms * 128 + (size_t)img_bytes);
}

size_t tc_smem_bytes(const TcArgs& a)
{
    return 1024 + (size_t)a.nstage * a.group * tc_stage_bytes(a.k_atoms, a.img_bytes, a.nprod) +
           (2 * TC_MAXSTAGE + 1) * sizeof(uint64_t) + 16;
}

// Dynamic shared memory a CTA may take: 227 KB less the kernel's static entry
// list (TC_MAXENT entries) and a reserve.
constexpr size_t TC_DYN_SMEM_MAX = 227 * 1024 - TC_MAXENT * sizeof(CEntry) - 512;

// Stages per CTA: at most about 100 KB of dynamic shared memory, so that two CTAs
// (with their static entry list and the per-CTA reserve) share an SM; at least 2
// where they fit.
int tc_pick_stages(int k_atoms, int img_bytes, int nprod)
{
    const size_t st = tc_stage_bytes(k_atoms, img_bytes, nprod);
    int ns = (int)((100 * 1024 - 1200) / st);
    if (ns < 2) ns = 2;
    if (ns > TC_MAXSTAGE) ns = TC_MAXSTAGE;
    while (ns > 1 && 1024 + ns * st + (2 * TC_MAXSTAGE + 1) * sizeof(uint64_t) + 16 > TC_DYN_SMEM_MAX) ns--;
    return ns;
}

int tc_max_stages(int k_atoms, int img_bytes, int nprod)
{
    const size_t st = tc_stage_bytes(k_atoms, img_bytes, nprod);
    int ns = TC_MAXSTAGE;
    while (ns > 1 && 1024 + ns * st + (2 * TC_MAXSTAGE + 1) * sizeof(uint64_t) + 16 > TC_DYN_SMEM_MAX) ns--;
    return ns;
}

void launch_m2l_tc(const TcArgs& a, int ntasks, cudaStream_t s, bool pdl)
{
    if (ntasks <= 0) return;
    size_t shm = tc_smem_bytes(a);
    static size_t attr = 0;
    if (shm > attr) {
        cudaFuncSetAttribute(k_m2l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        attr = shm;
    }
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    launch_k(k_m2l_tc, dim3(ntasks), dim3(TC_THREADS), shm, s, pdl, a);
}

}  // namespace gbfmm

namespace gbfmm {

// Batched launches of the grid conversion and the tensor-core M2L (one struct
// of arguments per system in device memory; the tensor maps are read there).
namespace {
__device__ __forceinline__ int tc_batch_system(const int* first, int nsys, int b)
{
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&first[mid]) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
}  // namespace

__global__ void __launch_bounds__(256) k_tc_grids_batch(const TcGridArgs* as, const int* first, int nsys)
{
    const int sys = tc_batch_system(first, nsys, (int)blockIdx.x);
    tc_grids_body(as[sys], (int)blockIdx.x - __ldg(&first[sys]));
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_m2l_tc_batch(const TcArgs* as, const int* first, int nsys)
{
    const int sys = tc_batch_system(first, nsys, (int)blockIdx.x);
    m2l_tc_body(as[sys], (int)blockIdx.x - __ldg(&first[sys]));
}

void launch_batch_tc(BatchKernel k, const void* args, const int* first, int nsys, int nblocks, size_t smem,
                     cudaStream_t s)
{
    if (nsys <= 0 || nblocks <= 0) return;
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    if (k == BatchKernel::TC_GRIDS) {
        k_tc_grids_batch<<<nblocks, 256, 0, s>>>((const TcGridArgs*)args, first, nsys);
    } else if (k == BatchKernel::M2L_TC) {
        static size_t attr = 0;
        if (smem > attr) {
            cudaFuncSetAttribute(k_m2l_tc_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            attr = smem;
        }
        k_m2l_tc_batch<<<nblocks, TC_THREADS, smem, s>>>((const TcArgs*)args, first, nsys);
    }
}

// Blocks of one system's grid conversion (and root L2L).
long tc_grids_blocks(const TcGridArgs& g)
{
    const long n = (g.rows - g.row_begin) * (g.KP / 8);
    if (n <= 0) return 0;
    return (n + 255) / 256 + (g.root_l2l ? ((long)g.root_n1 * g.root_R + 7) / 8 : 0);
}

}  // namespace gbfmm
