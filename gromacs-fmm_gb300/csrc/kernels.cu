// Device kernels of the GB300 FMM (sm_103a).
//
// Data layout in HBM:
//   atoms      float4 (u, q) per body in tree order; u = (x - leaf centre) / h_leaf
//   M, L       per level k: 8^k rows of Rpad floats (real (P+1)^2 representation,
//              scaled by the level's cell size h_k: M~_n = M_n/h^n, L~_j = L_j h^(j+1)),
//              rows indexed by Morton code
//   root       M~_0, L~_0 in FP64 (plus an FP32 copy of M~_0 for level-1 M2L)
//   field      float4 (phi, grad) per body in tree order, scaled units
#include <algorithm>
#include <cuda_runtime.h>

#include <atomic>

#include "async.cuh"
#include "common.cuh"
#include "kernels.h"

namespace gbfmm {

// Kernel launches issued by this library (all launch_* wrappers count theirs).
std::atomic<long> g_kernel_launches{0};
#define COUNT_LAUNCH() g_kernel_launches.fetch_add(1, std::memory_order_relaxed)

int sm_count()
{
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 1;
    }
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v <= 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
            cudaGetLastError();
            v = 1;
        }
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

// ------------------------------------------------------------------ tree

// Sum of per-block partials held as FP32 pairs (hi, lo) at part[stride * b] for
// b < nblocks, by one warp, in FP32-pair arithmetic (about 48 bits, the precision
// of the partials themselves): every load issued first (one round trip), each
// lane's blocks added in block order, then the fixed butterfly of f2s_warp_sum
// (every lane ends with the same sum), returned as an FP64 number.  Not FP64: an
// SM of this GPU retires two FP64 lanes per clock, and an FP64 sum of a few
// hundred partials by one CTA took microseconds on the step's serial path.
__device__ __forceinline__ double sum_partials(const float2* part, int stride, int nblocks)
{
    static_assert(TREE_MAX_BLOCKS == FINAL_MAX_BLOCKS, "one shape for both reductions");
    constexpr int K = (TREE_MAX_BLOCKS + 31) / 32;
    const int lane = threadIdx.x & 31;
    float2 p[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int b = lane + 32 * k;
        p[k] = b < nblocks ? __ldcg(&part[(size_t)stride * b]) : make_float2(0.f, 0.f);
    }
    f2sum t = {p[0].x, p[0].y};
#pragma unroll
    for (int k = 1; k < K; k++) t = f2s_add(t, f2sum{p[k].x, p[k].y});
    return f2s_value(f2s_warp_sum(t));
}

// Sum over the tree-key blocks of one of the four per-block partials (dipole x, y,
// z, total charge; FP32 pairs), by sum_partials.
__device__ __forceinline__ double sum_tree_partials(const double* partials, int nblocks, int quantity)
{
    return sum_partials(reinterpret_cast<const float2*>(partials) + quantity, 4, nblocks);
}

__device__ __forceinline__ void tree_keys_body(const TreeArgs& a, const int bid, const int nb)
{
    extern __shared__ float sh[];
    const int nd = 1 << a.depth;
    const StepConst* sc = a.sc;
    static_assert(sizeof(StepConst) % 8 == 0, "copied in 8-byte words");
    if (a.sc_copy && bid == 0) {
        // the constants (a kernel parameter) to the device copy that the later
        // kernels of the step read
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(sc);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(a.sc_copy);
        for (int i = threadIdx.x; i < (int)(sizeof(StepConst) / 8); i += blockDim.x) dst[i] = src[i];
    }
    float* th = sh;                                   // 3 x (nd+1)
    float2* ce = reinterpret_cast<float2*>(sh + ((3 * (nd + 1) + 1) & ~1));  // 3 x nd
    for (int i = threadIdx.x; i < 3 * (nd + 1); i += blockDim.x) th[i] = sc->thresh[i / (nd + 1)][i % (nd + 1)];
    for (int i = threadIdx.x; i < 3 * nd; i += blockDim.x) ce[i] = sc->centre[i / nd][i % nd];
    const float inv_h = sc->inv_h;
    const float* coords = sc->coords;
    const int ndv[3] = {sc->nd[0], sc->nd[1], sc->nd[2]};  // leaf cells per axis (nd, or nd / 2 across a slab)
    if (threadIdx.x == 0) {
        // L2 prefetch of the small operators and lists that the later stages
        // read: 4 KB chunks, spread over the blocks (one chunk list per array)
        for (int k = 0; k < TreeArgs::MAX_PREFETCH; k++) {
            const char* base = static_cast<const char*>(a.pf[k]);
            const unsigned long long bytes = a.pf_bytes[k] & ~15ull;
            const unsigned long long chunks = (bytes + 4095) >> 12;
            for (unsigned long long c = bid; c < chunks; c += nb) {
                const unsigned long long o = c << 12;
                const unsigned sz = (unsigned)min(4096ull, bytes - o);
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(base + o), "r"(sz) : "memory");
            }
        }
    }
    for (long i = (long)bid * blockDim.x + threadIdx.x; i < a.zero_n4; i += (long)nb * blockDim.x)
        a.zero[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    f2sum sd[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};  // dipole (3), total charge
    int bad = 0;
    for (int i = bid * blockDim.x + threadIdx.x; i < a.n; i += nb * blockDim.x) {
        float x[3] = {coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]};
        float q = a.charges[i];
        if (!isfinite(x[0]) || !isfinite(x[1]) || !isfinite(x[2]) || !isfinite(q)) bad = 1;
        int iv[3];
        float u[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const int ndd = ndv[d];
            float kf = fminf(fmaxf(x[d] * inv_h, 0.0f), (float)(ndd - 1));
            int k = (int)kf;
            const float* T = th + d * (nd + 1);
            // cell k holds T[k] < x <= T[k+1]: the strict '>' descent of tree.cpp:49-51
            while (k > 0 && !(x[d] > T[k])) k--;
            while (k < ndd - 1 && x[d] > T[k + 1]) k++;
            iv[d] = k;
            float2 c = ce[d * nd + k];
            u[d] = ((x[d] - c.x) - c.y) * inv_h;
        }
        uint32_t code = morton_encode(iv[0], iv[1], iv[2]);
        a.code[i] = code;
        a.uq[i] = make_float4(u[0], u[1], u[2], q);
        if (a.rank) a.rank[i] = atomicAdd(&a.counts[code], 1);
        else atomicAdd(&a.counts[code], 1);
#pragma unroll
        for (int d = 0; d < 3; d++) sd[d] = f2s_add(sd[d], f2s_prod(q, x[d]));
        sd[3] = f2s_add(sd[3], f2sum{q, 0.f});
    }
    // block reduction of the dipole and total charge (exact products, FP32-pair
    // sums in a fixed order)
    __shared__ f2sum red[8][4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const f2sum w = f2s_warp_sum(sd[k]);
        if (lane == 0) red[warp][k] = w;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        f2sum t = red[0][threadIdx.x];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) t = f2s_add(t, red[w][threadIdx.x]);
        reinterpret_cast<f2sum*>(a.partials)[4 * bid + threadIdx.x] = t;
    }
    if (bad) atomicOr(&a.flags[0], 1);
    if (!a.done) return;
    // last block: the leaf scan, and (when sums != NULL) the sums of the partials;
    // the solver leaves the sums to the upper-tree kernel, off this serial path
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(a.done, 1) == (int)nb - 1;
    __syncthreads();
    if (!s_last) return;
    pdl_trigger();  // the other blocks have exited: the scatter may launch
    __threadfence();
    if (threadIdx.x == 0) *a.done = 0;  // every block has counted: ready for the next step
    if (a.sums && warp < 4) {
        const double t = sum_tree_partials(a.partials, (int)nb, warp);
        if (lane == 0) a.sums[warp] = t;
    }
    if (a.off) {
        // exclusive scan of counts in tiles of 4096 staged in shared memory
        // (coalesced loads and stores); thread t scans 16 consecutive leaves
        __shared__ int4 tile4[1024];
        int* tile = reinterpret_cast<int*>(tile4);
        __shared__ int wsum[8];
        __shared__ int carry_s;
        const int n = a.nleaf;
        int carry = 0;
        for (int base = 0; base < n; base += 4096) {
            const int m = min(4096, n - base);
            for (int i = threadIdx.x; i < 4096; i += 256) tile[i] = i < m ? __ldcg(&a.counts[base + i]) : 0;
            __syncthreads();
            int c[16];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int4 v = tile4[4 * threadIdx.x + k];
                c[4 * k] = v.x;
                c[4 * k + 1] = v.y;
                c[4 * k + 2] = v.z;
                c[4 * k + 3] = v.w;
            }
            int t = 0;
#pragma unroll
            for (int k = 0; k < 16; k++) t += c[k];
            int x = t;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) wsum[warp] = x;
            __syncthreads();
            int run = carry + x - t;
            for (int w = 0; w < warp; w++) run += wsum[w];
#pragma unroll
            for (int k = 0; k < 16; k++) {
                const int v = run;
                run += c[k];
                c[k] = v;
            }
#pragma unroll
            for (int k = 0; k < 4; k++) tile4[4 * threadIdx.x + k] = make_int4(c[4 * k], c[4 * k + 1], c[4 * k + 2], c[4 * k + 3]);
            if (threadIdx.x == 255) carry_s = run;
            __syncthreads();
            for (int i = threadIdx.x; i < m; i += 256) {
                const int v = tile[i];
                a.off[base + i] = v;
                if (a.cursor) a.cursor[base + i] = v;
            }
            carry = carry_s;
            __syncthreads();  // the tile is reused by the next 4096 leaves
        }
        if (threadIdx.x == 0) a.off[n] = carry;
    }
}

__global__ void __launch_bounds__(256) k_tree_keys(TreeArgs a) { tree_keys_body(a, blockIdx.x, gridDim.x); }

int tree_blocks(int n) { return n <= 0 ? 1 : (n + 255) / 256 < TREE_MAX_BLOCKS ? (n + 255) / 256 : TREE_MAX_BLOCKS; }
int final_blocks(int n) { return n <= 0 ? 1 : (n + 255) / 256 < FINAL_MAX_BLOCKS ? (n + 255) / 256 : FINAL_MAX_BLOCKS; }

// The step's constants as a kernel parameter (copied with the launch, and in a
// CUDA graph updated on the node before each launch): the kernel reads them from
// the parameter space and block 0 stores them to a.sc_copy for the later kernels.
__global__ void __launch_bounds__(256) k_tree_keys_sc(TreeArgs a, const __grid_constant__ StepConst sc)
{
    a.sc = &sc;
    tree_keys_body(a, blockIdx.x, gridDim.x);
}

const void* tree_keys_sc_kernel() { return reinterpret_cast<const void*>(&k_tree_keys_sc); }

void launch_tree_keys(const TreeArgs& a, cudaStream_t s, const StepConst* by_value)
{
    int nd = 1 << a.depth;
    size_t shm = sizeof(float) * (((3 * (nd + 1) + 1) & ~1) + 6 * nd);
    int blocks = tree_blocks(a.n);
    COUNT_LAUNCH();
    if (by_value) k_tree_keys_sc<<<blocks, 256, shm, s>>>(a, *by_value);
    else k_tree_keys<<<blocks, 256, shm, s>>>(a);
}

// Exclusive scan of n ints (out[n] = total), three phases of 2048-element blocks.
__global__ void __launch_bounds__(512) k_scan_blocks(const int* in, int* out, int n, int* bsum)
{
    __shared__ int ws[16];
    const int base = blockIdx.x * 2048 + threadIdx.x * 4;
    int v[4], t = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        v[i] = base + i < n ? in[base + i] : 0;
        t += v[i];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = t;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < 16 ? ws[lane] : 0;
        for (int o = 1; o < 16; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < 16) ws[lane] = w;
    }
    __syncthreads();
    int excl = x - t + (warp > 0 ? ws[warp - 1] : 0);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        if (base + i < n) out[base + i] = excl;
        excl += v[i];
    }
    if (threadIdx.x == 511) bsum[blockIdx.x] = excl;
}

__global__ void __launch_bounds__(1024) k_scan_top(int* bsum, int nb, int* total)
{
    __shared__ int ws[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int carry = 0;
    for (int base = 0; base < nb; base += 1024) {
        int i = base + threadIdx.x;
        int v = i < nb ? bsum[i] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int w = ws[lane];
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            ws[lane] = w;
        }
        __syncthreads();
        int incl = x + (warp > 0 ? ws[warp - 1] : 0);
        if (i < nb) bsum[i] = carry + incl - v;
        int blocktotal = ws[31];
        __syncthreads();
        carry += blocktotal;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int* out, int n, const int* bsum)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += bsum[i / 2048];
}

void launch_exclusive_scan(const int* in, int* out, int n, int* scratch, cudaStream_t s)
{
    int nb = (n + 2047) / 2048;
    COUNT_LAUNCH();
    k_scan_blocks<<<nb, 512, 0, s>>>(in, out, n, scratch);
    COUNT_LAUNCH();
    k_scan_top<<<1, 1024, 0, s>>>(scratch, nb, out + n);
    if (nb > 1) { COUNT_LAUNCH(); k_scan_add<<<(n + 255) / 256, 256, 0, s>>>(out, n, scratch); }
}

__global__ void k_scatter(const uint32_t* code, int n, int* cursor, int* tmp_idx)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) tmp_idx[atomicAdd(&cursor[code[i]], 1)] = i;
}

void launch_scatter(const uint32_t* code, int n, int* cursor, int* tmp_idx, cudaStream_t s)
{
    if (n > 0) { COUNT_LAUNCH(); k_scatter<<<(n + 255) / 256, 256, 0, s>>>(code, n, cursor, tmp_idx); }
}

__device__ __forceinline__ void scatter_ranked_body(const ScatterArgs& a, const int bid)
{
    pdl_wait();
    pdl_trigger();
    int i = bid * blockDim.x + threadIdx.x;
    if (i < a.n) a.tmp[a.off[a.code[i]] + a.rank[i]] = i;
}

__global__ void k_scatter_ranked(const ScatterArgs a) { scatter_ranked_body(a, blockIdx.x); }

void launch_scatter_ranked(const uint32_t* code, int n, const int* off, const int* rank, int* tmp_idx,
                           cudaStream_t s, bool pdl)
{
    if (n > 0) {
        COUNT_LAUNCH();
        ScatterArgs a{code, n, off, rank, tmp_idx};
        launch_k(k_scatter_ranked, dim3((n + 255) / 256), dim3(256), 0, s, pdl, a);
    }
}

// Stable order inside each leaf (ascending input index), which makes the body
// order identical to the per-level stable counting sort of tree.cpp:43-74.
// A body on or near a face of its leaf, or outside it (|u| >= 1/2 - 2^-20 in
// scaled units): the near field then takes the r = 0 test on every pair.
__device__ __forceinline__ bool at_leaf_face(float4 b)
{
    return fmaxf(fabsf(b.x), fmaxf(fabsf(b.y), fabsf(b.z))) >= 0.5f - 0x1p-20f;
}

__device__ __forceinline__ void leaf_sort_body(const LeafSortArgs& la, const int bid)
{
    const int* off = la.off;
    const int nleaf = la.nleaf;
    const int* tmp_idx = la.tmp_idx;
    const float4* uq = la.uq;
    int* order = la.order;
    float4* atoms = la.atoms;
    int* inv = la.inv;
    int* counts = la.counts;
    int* edge = la.edge;
    const int lane = threadIdx.x & 31;
    const int leaf = (bid * blockDim.x + threadIdx.x) >> 5;
    pdl_wait();
    pdl_trigger();
    if (leaf >= nleaf) return;
    if (counts && lane == 0) counts[leaf] = 0;  // consumed by the scan: zero for the next step
    const int b = off[leaf], n = off[leaf + 1] - b;
    bool face = false;
    if (n <= 32) {
        int v = lane < n ? tmp_idx[b + lane] : 0x7fffffff;
        int rank = 0;
        for (int j = 0; j < 32; j++) {
            int w = __shfl_sync(0xffffffffu, v, j);
            rank += (w < v);
        }
        if (lane < n) {
            order[b + rank] = v;
            const float4 a = uq[v];
            atoms[b + rank] = a;
            inv[v] = b + rank;
            face = at_leaf_face(a);
        }
    } else {
        for (int e = lane; e < n; e += 32) {
            int v = tmp_idx[b + e];
            int rank = 0;
            for (int j = 0; j < n; j++) rank += (tmp_idx[b + j] < v);
            order[b + rank] = v;
            const float4 a = uq[v];
            atoms[b + rank] = a;
            inv[v] = b + rank;
            face |= at_leaf_face(a);
        }
    }
    const unsigned any = __ballot_sync(0xffffffffu, face);
    if (edge && lane == 0) edge[leaf] = any != 0u;
}

__global__ void __launch_bounds__(256) k_leaf_sort(const LeafSortArgs a) { leaf_sort_body(a, blockIdx.x); }

void launch_leaf_sort(const int* offsets, int nleaf, int* tmp_idx, const float4* uq, const uint32_t* code, int* order,
                      float4* atoms, int* inv, int* counts, cudaStream_t s, int* edge, bool pdl)
{
    (void)code;
    long threads = (long)nleaf * 32;
    COUNT_LAUNCH();
    LeafSortArgs a{offsets, nleaf, tmp_idx, uq, order, atoms, inv, counts, edge};
    launch_k(k_leaf_sort, dim3((unsigned)((threads + 255) / 256)), dim3(256), 0, s, pdl, a);
}

// ------------------------------------------------------------------ P2M

// Streams the regular harmonics Y_n^m(u), m >= 0, in (m outer, n inner) order and
// calls f(n, m, re, im) for each.  Recurrences (exafmm normalisation):
//   Y_m^m = Y_{m-1}^{m-1} (x+iy) / (2m),  Y_{m+1}^m = -z Y_m^m,
//   Y_{n+1}^m = -((2n+1) z Y_n^m + r^2 Y_{n-1}^m) / ((n+m+1)(n-m+1)).
template <int P, typename F>
__device__ __forceinline__ void stream_regular(float x, float y, float z, F&& f)
{
    // Every product and fused multiply-add is spelled out (no contraction left
    // to the compiler), so that each kernel that inlines this recurrence, the
    // single-system and the batched instances alike, rounds it the same way.
    const float r2 = fmaf(x, x, fmaf(y, y, __fmul_rn(z, z)));
    float sr = 1.f, si = 0.f;
#pragma unroll
    for (int m = 0; m <= P; m++) {
        if (m > 0) {
            const float inv = 1.0f / (2 * m);
            float tr = __fmul_rn(fmaf(sr, x, -__fmul_rn(si, y)), inv);
            float ti = __fmul_rn(fmaf(sr, y, __fmul_rn(si, x)), inv);
            sr = tr;
            si = ti;
        }
        f(m, m, sr, si);
        if (m + 1 <= P) {
            float ar = sr, ai = si;          // Y_{n-1}
            float br = -z * sr, bi = -z * si;  // Y_n
            f(m + 1, m, br, bi);
#pragma unroll
            for (int n = m + 1; n < P; n++) {
                const float c = 1.0f / ((n + m + 1) * (n - m + 1));
                const float kz = __fmul_rn((float)(2 * n + 1), z);
                float cr = -__fmul_rn(fmaf(kz, br, __fmul_rn(r2, ar)), c);
                float ci = -__fmul_rn(fmaf(kz, bi, __fmul_rn(r2, ai)), c);
                f(n + 1, m, cr, ci);
                ar = br; ai = bi;
                br = cr; bi = ci;
            }
        }
    }
}

template <int P, int WARPS>
__device__ __forceinline__ void p2m_body(const P2MArgs& pa, const int bid)
{
    constexpr int R = (P + 1) * (P + 1);
    constexpr int LD = 33;
    extern __shared__ float sm[];
    const int* off = pa.off;
    const int nleaf = pa.nleaf;
    const float4* atoms = pa.atoms;
    float* M = pa.M;
    const int Rpad = pa.Rpad;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int leaf = bid * WARPS + warp;
    pdl_wait();
    pdl_trigger();
    if (leaf >= nleaf) return;
    float* S = sm + warp * R * LD;
    for (int r = 0; r < R; r++) S[r * LD + lane] = 0.f;
    const int b = off[leaf], n = off[leaf + 1] - b;
    for (int c0 = 0; c0 < n; c0 += 32) {
        float4 a = c0 + lane < n ? atoms[b + c0 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float q = a.w;
        // M~ += q conj(Y(u)), kernel.cu:228-240 evaluated at -phi
        stream_regular<P>(a.x, a.y, a.z, [&](int nn, int mm, float yr, float yi) {
            float* sre = &S[ridx_re(nn, mm) * LD + lane];
            *sre = fmaf(q, yr, *sre);
            if (mm > 0) {
                float* sim = &S[ridx_im(nn, mm) * LD + lane];
                *sim = fmaf(-q, yi, *sim);
            }
        });
    }
    __syncwarp();
    float* out = M + (long)leaf * Rpad;
    for (int r = lane; r < R; r += 32) {
        float t = 0.f;
#pragma unroll 8
        for (int c = 0; c < 32; c++) t += S[r * LD + c];
        out[r] = t;
    }
}

template <int P, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_p2m(const P2MArgs a) { p2m_body<P, WARPS>(a, blockIdx.x); }

template <int P>
static void p2m_dispatch(const int* off, int nleaf, const float4* atoms, float* M, int Rpad, cudaStream_t s, bool pdl)
{
    constexpr int R = (P + 1) * (P + 1);
    constexpr int W = R <= 169 ? 4 : 2;
    size_t shm = sizeof(float) * W * R * 33;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_p2m<P, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        attr = true;
    }
    COUNT_LAUNCH();
    P2MArgs a{off, nleaf, atoms, M, nullptr, nullptr, Rpad};
    launch_k(k_p2m<P, W>, dim3((nleaf + W - 1) / W), dim3(W * 32), shm, s, pdl, a);
}

#define GBFMM_ORDER_SWITCH(P, CALL)            \
    switch (P) {                              \
        case 2: { constexpr int PP = 2; CALL; } break;   \
        case 3: { constexpr int PP = 3; CALL; } break;   \
        case 4: { constexpr int PP = 4; CALL; } break;   \
        case 5: { constexpr int PP = 5; CALL; } break;   \
        case 6: { constexpr int PP = 6; CALL; } break;   \
        case 7: { constexpr int PP = 7; CALL; } break;   \
        case 8: { constexpr int PP = 8; CALL; } break;   \
        case 9: { constexpr int PP = 9; CALL; } break;   \
        case 10: { constexpr int PP = 10; CALL; } break; \
        case 11: { constexpr int PP = 11; CALL; } break; \
        case 12: { constexpr int PP = 12; CALL; } break; \
        case 13: { constexpr int PP = 13; CALL; } break; \
        case 14: { constexpr int PP = 14; CALL; } break; \
        case 15: { constexpr int PP = 15; CALL; } break; \
        case 16: { constexpr int PP = 16; CALL; } break; \
        default: break;                       \
    }

void launch_p2m(int P, const int* offsets, int nleaf, const float4* atoms, float* M_leaf, int Rpad, cudaStream_t s,
                bool pdl)
{
    GBFMM_ORDER_SWITCH(P, p2m_dispatch<PP>(offsets, nleaf, atoms, M_leaf, Rpad, s, pdl));
}

// ------------------------------------------------------------------ L2P

// phi = sum_n [Re(L_n0 Y_n0) + 2 sum_{m>0} Re(L_nm Y_nm)], the L2P sum of kernel.cu:635-651,
// and its Cartesian gradient from the ladder identities
//   dz Y_nm = -Y_{n-1,m};  (dx+i dy) Y_nm = -Y_{n-1,m+1};
//   (dx-i dy) Y_nm = Y_{n-1,m-1} (m>0),  (dx-i dy) Y_n0 = -conj(Y_{n-1,1}).
template <int P, int WARPS>
__device__ __forceinline__ void l2p_body(const L2PArgs& la, const int bid)
{
    constexpr int R = (P + 1) * (P + 1);
    __shared__ float Ls[WARPS][R + 1];
    const int* off = la.off;
    const int nleaf = la.nleaf;
    const float4* atoms = la.atoms;
    const float* L = la.L;
    const int Rpad = la.Rpad;
    float4* field = la.field;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int leaf = bid * WARPS + warp;
    if (leaf >= nleaf) return;
    const float* src = L + (long)leaf * Rpad;
    float* Lw = Ls[warp];
    for (int r = lane; r < R; r += 32) Lw[r] = src[r];
    __syncwarp();
    const int b = off[leaf], n = off[leaf + 1] - b;
    auto lre = [&](int nn, int mm) { return Lw[ridx_re(nn, mm)]; };
    auto lim = [&](int nn, int mm) { return mm > 0 ? Lw[ridx_im(nn, mm)] : 0.f; };
    for (int c0 = 0; c0 < n; c0 += 32) {
        if (c0 + lane >= n) break;
        const float4 a = atoms[b + c0 + lane];
        float phi = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
        stream_regular<P>(a.x, a.y, a.z, [&](int np, int mp, float ya, float yb) {
            const float wm = mp == 0 ? 1.f : 2.f;
            phi += wm * (lre(np, mp) * ya - lim(np, mp) * yb);
            if (np + 1 <= P) {
                float Lr = lre(np + 1, mp), Li = lim(np + 1, mp);
                gz -= wm * (Lr * ya - Li * yb);
                if (mp >= 1) {
                    const float w = (mp - 1) == 0 ? 1.f : 2.f;
                    Lr = lre(np + 1, mp - 1);
                    Li = lim(np + 1, mp - 1);
                    gx -= 0.5f * w * (Lr * ya - Li * yb);
                    gy -= 0.5f * w * (Lr * yb + Li * ya);
                }
                Lr = lre(np + 1, mp + 1);
                Li = lim(np + 1, mp + 1);
                gx += (Lr * ya - Li * yb);
                gy -= (Lr * yb + Li * ya);
                if (mp == 1) {
                    Lr = lre(np + 1, 0);
                    gx -= 0.5f * Lr * ya;
                    gy -= 0.5f * Lr * yb;
                }
            }
        });
        field[b + c0 + lane] = make_float4(phi, gx, gy, gz);
    }
}

template <int P, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_l2p(const L2PArgs a) { l2p_body<P, WARPS>(a, blockIdx.x); }

void launch_l2p(int P, const int* offsets, int nleaf, const float4* atoms, const float* L_leaf, int Rpad,
                float4* field, cudaStream_t s)
{
    COUNT_LAUNCH();
    L2PArgs a{offsets, nleaf, atoms, L_leaf, Rpad, field};
    GBFMM_ORDER_SWITCH(P, (k_l2p<PP, 4><<<(nleaf + 3) / 4, 128, 0, s>>>(a)));
}

// ------------------------------------------------------------------ fused downward pass

__device__ __forceinline__ int real_degree(int r) { return (int)sqrtf((float)r + 0.5f); }

// Orders whose 8 L2L operators (32 (P+1)^4 bytes) the downward pass stages in
// shared memory: up to 6 (76.8 KB).
#define DOWN_STAGE(P) (32 * (P + 1) * (P + 1) * (P + 1) * (P + 1) <= 80 * 1024)

// Downward pass in one launch.  CTA = one leaf-parent cell p (level D-1, D >= 2):
// the locals of p's ancestors are rebuilt from level 1 down (L~_k = M2L part + L2L
// of the parent, in the order of the one-level kernels: a few R^2 FMAs each, the
// same for every CTA of the subtree), then p's 8 leaves, then L2P of their bodies
// (one warp per leaf).
template <int P>
__device__ __forceinline__ void down_body(const DownArgs& a, const int bid)
{
    constexpr int R = (P + 1) * (P + 1);
    // the 8 operators in shared memory (one bulk copy) where they fit: every
    // L2L below reads them R times per row
    constexpr bool STAGED = DOWN_STAGE(P);
    extern __shared__ float4 dsm4[];
    __shared__ uint64_t dbar;
    __shared__ float Lanc[MAX_DEPTH][R];  // the ancestors' rows (levels 1..D-1)
    __shared__ float Lbuf[2][R];
    __shared__ float Lleaf[8][R + 1];
    const int D = a.depth;
    const uint32_t p = bid;
    const float* At = a.l2l_t;
    if constexpr (STAGED) {
        float* sA = reinterpret_cast<float*>(dsm4);
        if (threadIdx.x == 0) {
            mbar_init(&dbar, 1);
            mbar_init_fence();
            mbar_expect_tx(&dbar, 32u * R * R);
            bulk_g2s(sA, a.l2l_t, 32u * R * R, &dbar);  // constant: may precede the wait below
        }
        At = sA;
    }
    pdl_wait();
    // every local row the CTA reads, in one pass: the ancestors' (level k's
    // ancestor of parent p is p >> 3 (D-1-k)) and the 8 leaves'
    for (int i = threadIdx.x; i < (D + 7) * R; i += blockDim.x) {
        const int k = 1 + i / R, r = i % R;
        if (k < D) {
            const uint32_t anc = p >> (3 * (D - 1 - k));
            Lanc[k - 1][r] = a.L[k][(size_t)anc * a.Rpad + r];
        } else {
            const int o = k - D;
            Lleaf[o][r] = a.L[D][(size_t)((p << 3) | (uint32_t)o) * a.Rpad + r];
        }
    }
    __syncthreads();
    if constexpr (STAGED) {
        // on a give-up the kernel waits (bounded) for the copy before reading on
        if (!mbar_wait(&dbar, 0, a.err, 1, a.wait_limit)) mbar_drain(&dbar, 0, a.wait_limit);
    }
    // L2L down the ancestors: each output row's dot product split over 4
    // consecutive lanes (columns c = j^2 + q, + 4, ...), added by a fixed butterfly
    const float* Lc = Lanc[0];
    for (int k = 2; k <= D - 1; k++) {
        const uint32_t anc = p >> (3 * (D - 1 - k));
        const float* A0 = At + (size_t)(anc & 7) * R * R;
        float* Ln = Lbuf[k & 1];
        for (int base = 0; base < 4 * R; base += blockDim.x) {
            const int w = base + threadIdx.x;
            const bool act = w < 4 * R;
            const int r = act ? w >> 2 : 0, q = w & 3;
            float acc = 0.f;
            if (act) {
                const int j = real_degree(r);
                for (int c = j * j + q; c < R; c += 4) acc = fmaf(A0[(size_t)c * R + r], Lc[c], acc);
            }
            acc += __shfl_xor_sync(0xffffffffu, acc, 1);
            acc += __shfl_xor_sync(0xffffffffu, acc, 2);
            if (act && q == 0) Ln[r] = Lanc[k - 1][r] + acc;
        }
        __syncthreads();
        Lc = Ln;
    }
    // the 8 leaves: their M2L part (preloaded) plus the L2L of the parent
    for (int i = threadIdx.x; i < 8 * R; i += blockDim.x) {
        const int o = i / R, r = i - o * R;
        const float* A0 = At + (size_t)o * R * R;
        const int j = real_degree(r);
        float acc = 0.f;
        for (int c = j * j; c < R; c++) acc = fmaf(A0[(size_t)c * R + r], Lc[c], acc);
        Lleaf[o][r] += acc;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, o = threadIdx.x >> 5;
    const uint32_t leaf = (p << 3) | (uint32_t)o;
    const float* Lw = Lleaf[o];
    auto lre = [&](int nn, int mm) { return Lw[ridx_re(nn, mm)]; };
    auto lim = [&](int nn, int mm) { return mm > 0 ? Lw[ridx_im(nn, mm)] : 0.f; };
    const int b = a.off[leaf], n = a.off[leaf + 1] - b;
    for (int c0 = 0; c0 < n; c0 += 32) {
        if (c0 + lane >= n) break;
        const float4 q = a.atoms[b + c0 + lane];
        float phi = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
        stream_regular<P>(q.x, q.y, q.z, [&](int np, int mp, float ya, float yb) {
            const float wm = mp == 0 ? 1.f : 2.f;
            phi += wm * (lre(np, mp) * ya - lim(np, mp) * yb);
            if (np + 1 <= P) {
                float Lr = lre(np + 1, mp), Li = lim(np + 1, mp);
                gz -= wm * (Lr * ya - Li * yb);
                if (mp >= 1) {
                    const float w = (mp - 1) == 0 ? 1.f : 2.f;
                    Lr = lre(np + 1, mp - 1);
                    Li = lim(np + 1, mp - 1);
                    gx -= 0.5f * w * (Lr * ya - Li * yb);
                    gy -= 0.5f * w * (Lr * yb + Li * ya);
                }
                Lr = lre(np + 1, mp + 1);
                Li = lim(np + 1, mp + 1);
                gx += (Lr * ya - Li * yb);
                gy -= (Lr * yb + Li * ya);
                if (mp == 1) {
                    Lr = lre(np + 1, 0);
                    gx -= 0.5f * Lr * ya;
                    gy -= 0.5f * Lr * yb;
                }
            }
        });
        a.field[b + c0 + lane] = make_float4(phi, gx, gy, gz);
    }
}

template <int P>
__global__ void __launch_bounds__(256) k_down(const DownArgs a) { down_body<P>(a, blockIdx.x); }

size_t down_smem_bytes(int P)
{
    const size_t R = (size_t)(P + 1) * (P + 1);
    return DOWN_STAGE(P) ? 32 * R * R : 0;
}

template <int P>
static void down_dispatch(const DownArgs& a, cudaStream_t s, bool pdl)
{
    const size_t shm = down_smem_bytes(P);
    static bool attr = false;
    if (!attr && shm > 0) {
        cudaFuncSetAttribute(k_down<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        attr = true;
    }
    launch_k(k_down<P>, dim3(a.nparent), dim3(256), shm, s, pdl, a);
}

void launch_down(int P, const DownArgs& a, cudaStream_t s, bool pdl)
{
    COUNT_LAUNCH();
    GBFMM_ORDER_SWITCH(P, down_dispatch<PP>(a, s, pdl));
}


// ------------------------------------------------------------------ P2P

constexpr int P2P_THREADS = 128;
constexpr int P2P_MAXS = 2048;  // staged source bodies per pass
constexpr int P2P_MAXT = 128;   // targets per pass

// 1/sqrt(x) by the PTX approximate instruction (relative error below 2^-22.9),
// denormal inputs flushed to zero.
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Packed FP32 pairs (PTX .f32x2, sm_100 and later): two lanes of FP32 work per
// instruction.  A b64 register holds (a, b).
typedef unsigned long long f2_t;
__device__ __forceinline__ f2_t f2_pack(float a, float b)
{
    f2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2_t v, float& a, float& b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b)
{
    f2_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b)
{
    f2_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b)
{
    f2_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c)
{
    f2_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Staged sources, two per record: {x_a, x_b, y_a, y_b}, {z_a, z_b, q_a, q_b}.
// Padding sources sit far away (1e15, scaled units) with zero charge, so that
// they add exact zeros without a test.
constexpr float P2P_FAR = 1e15f;

// K targets per thread against this warp's source steps [sb, se); a step holds
// SL source records (two sources each) and lane jj < SL takes record SL st + jj,
// two sources per packed instruction.  Pair term as kernel.cu:480-490:
// phi += q/r, grad += q (x_j - x_i)/r^3, skipped when r = 0 (a body with itself
// or a coincident body) where MASK is set.  Accumulates +q (x_i - x_j)/r^3; the
// caller negates.
template <int K, bool MASK, int SL>
__device__ __forceinline__ void p2p_sweep(const float4* __restrict__ src, int sb, int se, int jj, const f2_t (&X)[K][3],
                                          f2_t (&acc)[K][4])
{
#pragma unroll 2
    for (int st = sb; st < se; st++) {
        const float4 xy = src[2 * (SL * st + jj)];
        const float4 zq = src[2 * (SL * st + jj) + 1];
        const f2_t sx = f2_pack(xy.x, xy.y), sy = f2_pack(xy.z, xy.w), sz = f2_pack(zq.x, zq.y);
        const f2_t sq = f2_pack(zq.z, zq.w);
#pragma unroll
        for (int k = 0; k < K; k++) {
            const f2_t dx = f2_sub(X[k][0], sx), dy = f2_sub(X[k][1], sy), dz = f2_sub(X[k][2], sz);
            const f2_t r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_mul(dz, dz)));
            float ra, rb;
            f2_unpack(r2, ra, rb);
            float ia = rsqrt_approx(ra), ib = rsqrt_approx(rb);
            if (MASK) {
                ia = ra > 0.f ? ia : 0.f;
                ib = rb > 0.f ? ib : 0.f;
            }
            const f2_t ri = f2_pack(ia, ib);
            const f2_t qr = f2_mul(sq, ri);
            acc[k][0] = f2_add(acc[k][0], qr);
            const f2_t q3 = f2_mul(qr, f2_mul(ri, ri));
            acc[k][1] = f2_fma(q3, dx, acc[k][1]);
            acc[k][2] = f2_fma(q3, dy, acc[k][2]);
            acc[k][3] = f2_fma(q3, dz, acc[k][3]);
        }
    }
}

// One cluster of up to LT K targets starting at c0 (of this pass's ntc): lane =
// (target row ii = lane / SL, source lane jj = lane % SL), SL = 32 / LT; thread
// targets c0 + ii + LT k.  Steps below msteps need the r = 0 test.
template <int K, int LT>
// Target positions come from the staged records when tsm is set (the targets
// are the first bodies of window 0, the target leaf's own, unshifted), else
// from the sorted atoms.
__device__ __forceinline__ void p2p_cluster(const float4* __restrict__ src, const float4* __restrict__ tgt,
                                            const float* tsm, int c0, int ntc, int sb, int se, int msteps, int lane,
                                            float4* part)
{
    constexpr int SL = 32 / LT;
    const int ii = lane / SL, jj = lane % SL;
    f2_t X[K][3];
    f2_t acc[K][4];
    const f2_t zero = f2_pack(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int t = min(c0 + ii + LT * k, ntc - 1);
        float x, y, z;
        if (tsm) {
            const float* rec = tsm + 8 * (t >> 1) + (t & 1);
            x = rec[0];
            y = rec[2];
            z = rec[4];
        } else {
            const float4 a = tgt[t];
            x = a.x;
            y = a.y;
            z = a.z;
        }
        X[k][0] = f2_pack(x, x);
        X[k][1] = f2_pack(y, y);
        X[k][2] = f2_pack(z, z);
        acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = zero;
    }
    const int mid = min(max(msteps, sb), se);
    p2p_sweep<K, true, SL>(src, sb, mid, jj, X, acc);
    p2p_sweep<K, false, SL>(src, mid, se, jj, X, acc);
#pragma unroll
    for (int k = 0; k < K; k++) {
        float v[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float a, b;
            f2_unpack(acc[k][c], a, b);
            v[c] = a + b;
        }
        // fixed butterfly over the SL source lanes of each target
#pragma unroll
        for (int o = 1; o < SL; o <<= 1)
#pragma unroll
            for (int c = 0; c < 4; c++) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
        const int t = c0 + ii + LT * k;
        if (jj == 0 && t < ntc) {
            float4 pp = part[t];
            pp.x += v[0];
            pp.y -= v[1];
            pp.z -= v[2];
            pp.w -= v[3];
            part[t] = pp;
        }
    }
}

struct P2PShared {
    float4 src[P2P_MAXS];      // P2P_MAXS sources in P2P_MAXS/2 records of two float4
    float4 part[4][P2P_MAXT];  // per-warp partial sums, reduced in warp order
    int e_off[129];            // window position of each stencil leaf (even), and the total
    int e_beg[128];            // first body of the leaf in the sorted atoms
    int e_cnt[128];            // its body count
    char4 e_d[128];            // its stencil offset
    int ws[4];
    uint64_t bar;              // completion of the bulk copies of one window
    uint8_t tag[P2P_MAXS / 2]; // stencil leaf of each body pair of the window
};

// Initialises the staging barrier of a CTA (before its first p2p_leaf).
__device__ __forceinline__ void p2p_init(P2PShared& sh)
{
    if (threadIdx.x == 0) {
        mbar_init(&sh.bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
}

// The near field of one target leaf (the CTA's 128 threads).  The source bodies
// of the 81 near leaves are staged in shared memory in windows of P2P_MAXS
// bodies, each leaf at an even window position (an odd count leaves one far,
// chargeless padding body): one bulk copy per leaf (its bodies are contiguous in
// tree order, 16 bytes each) on an mbarrier, then, in place, every pair of
// bodies of a leaf becomes one record of two float4 shifted into the target
// leaf's frame (scaled units, integer offsets of the stencil, so the periodic
// shift is exact); the target leaf itself is staged first (stencil entry 0).  A
// warp step covers LT targets x SL = 32/LT source records; a thread carries up to
// KM targets (clusters of KM LT).  Warp w sweeps a quarter of the sources; the SL
// source lanes of a target are reduced by shuffles and the per-warp partial sums
// are added in warp order (deterministic).
//
// The r = 0 test is applied to the target leaf's own bodies only.  Bodies of two
// different leaves cannot coincide when every staged body lies strictly inside
// its leaf (|u| < 1/2 - 2^-20 in scaled units: the rounding of u and of the
// integer shift is far below that margin); a CTA whose stencil holds any leaf
// with a body outside that range (bodies on or near a leaf face, or outside the
// box; flagged per leaf by the leaf sort) applies the test to every source.
//
// 'phase' is the parity of the staging barrier's current phase (the same in
// every thread); a bounded wait that gives up sets bit 2 of *a.err.
template <int LT, int KM = 3>
__device__ __forceinline__ void p2p_leaf(const P2PArgs& a, uint32_t tcode, P2PShared& sh, uint32_t& phase)
{
    constexpr int SL = 32 / LT, SPS = 2 * SL;  // sources per step
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int tx, ty, tz;
    morton_decode(tcode, tx, ty, tz);
    const int tb = a.off[tcode], nt = a.off[tcode + 1] - tb;
    // source leaves of the stencil (their loads overlap the target leaf's)
    int cnt = 0, eflag = 0;
    if (tid < a.nst) {
        int vx = tx + a.stencil[3 * tid], vy = ty + a.stencil[3 * tid + 1], vz = tz + a.stencil[3 * tid + 2];
        bool ok = true;
        if (a.periodic) {
            vx &= a.nd[0] - 1; vy &= a.nd[1] - 1; vz &= a.nd[2] - 1;
        } else {
            ok = vx >= 0 && vy >= 0 && vz >= 0 && vx < a.nd[0] && vy < a.nd[1] && vz < a.nd[2];
        }
        if (ok) {
            uint32_t sc = morton_encode(vx, vy, vz);
            sh.e_beg[tid] = a.off[sc];
            cnt = a.off[sc + 1] - a.off[sc];
            eflag = a.leaf_edge[sc];
        } else {
            sh.e_beg[tid] = 0;
        }
        sh.e_cnt[tid] = cnt;
        sh.e_d[tid] = make_char4((signed char)a.stencil[3 * tid], (signed char)a.stencil[3 * tid + 1],
                                 (signed char)a.stencil[3 * tid + 2], 0);
    }
    if (nt == 0) return;  // uniform over the CTA
    // exclusive prefix of the even-rounded counts over the stencil entries (nst <= 128);
    // entries past nst have no bodies, so every thread from nst on writes the total
    {
        const int c2 = (cnt + 1) & ~1;
        int x = c2;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) sh.ws[warp] = x;
        __syncthreads();
        int add = 0;
        for (int w = 0; w < warp; w++) add += sh.ws[w];
        sh.e_off[tid] = x - c2 + add;
        if (tid == 0 && a.nst == P2P_THREADS) sh.e_off[a.nst] = sh.ws[0] + sh.ws[1] + sh.ws[2] + sh.ws[3];
    }
    // any staged leaf (the target leaf included: a target outside its leaf can
    // meet the image of a body well inside another leaf) with a body at a face:
    // then every pass takes the r = 0 test (flags from the leaf sort)
    const bool any_edge = __syncthreads_or(eflag) != 0;
    const int total = sh.e_off[a.nst], nself = sh.e_off[1];
    float* srcf = reinterpret_cast<float*>(sh.src);
    for (int t0 = 0; t0 < nt; t0 += P2P_MAXT) {
        const int ntc = min(P2P_MAXT, nt - t0);
        const float4* tgt = a.atoms + tb + t0;
        for (int i = tid; i < 4 * P2P_MAXT; i += P2P_THREADS)
            sh.part[i / P2P_MAXT][i % P2P_MAXT] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int s0 = 0; s0 < total; s0 += P2P_MAXS) {
            const int ns = min(P2P_MAXS, total - s0);
            const int nsp = (ns + SPS - 1) / SPS * SPS;
            __syncthreads();  // the previous window's readers are done
            // one bulk copy per stencil leaf: its bodies inside this window; and
            // the leaf's tag on each of its body pairs in the window
            if (tid < a.nst) {
                const int q0 = max(sh.e_off[tid], s0), q1 = min(sh.e_off[tid + 1], s0 + ns);
                for (int g = q0; g < q1; g += 2) sh.tag[(g - s0) >> 1] = (uint8_t)tid;
                const int b0 = max(sh.e_off[tid], s0), b1 = min(sh.e_off[tid] + sh.e_cnt[tid], s0 + ns);
                if (b1 > b0) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("mbarrier.expect_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&sh.bar)),
                                 "r"((uint32_t)(16 * (b1 - b0)))
                                 : "memory");
                    bulk_g2s(sh.src + (b0 - s0), a.atoms + sh.e_beg[tid] + (b0 - sh.e_off[tid]),
                             (uint32_t)(16 * (b1 - b0)), &sh.bar);
                }
            }
            __syncthreads();  // every expected byte count is on the barrier
            if (tid == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&sh.bar)) : "memory");
            if (!mbar_wait(&sh.bar, phase, a.err, 2, a.wait_limit)) mbar_drain(&sh.bar, phase, a.wait_limit);
            phase ^= 1u;
            // records, in place: thread t turns the body pairs t, t + 128, ... (each
            // within one stencil leaf: the leaves start at even positions)
            for (int pr = tid; pr < (ns >> 1); pr += P2P_THREADS) {
                const int e = sh.tag[pr];
                const int r = 2 * pr, g = s0 + r, real = sh.e_off[e] + sh.e_cnt[e];
                const char4 dc = sh.e_d[e];
                const float dx = (float)dc.x, dy = (float)dc.y, dz = (float)dc.z;
                const bool sa = g < real, sb = g + 1 < real;
                const float4 ba = sa ? sh.src[r] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 bb = sb ? sh.src[r + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
                sh.src[r] = make_float4(sa ? ba.x + dx : P2P_FAR, sb ? bb.x + dx : P2P_FAR, sa ? ba.y + dy : P2P_FAR,
                                        sb ? bb.y + dy : P2P_FAR);
                sh.src[r + 1] = make_float4(sa ? ba.z + dz : P2P_FAR, sb ? bb.z + dz : P2P_FAR, ba.w, bb.w);
            }
            // far zero-charge padding of the last step
            if (tid < (nsp - ns) / 2) {
                const int r = ns + 2 * tid;
                sh.src[r] = make_float4(P2P_FAR, P2P_FAR, P2P_FAR, P2P_FAR);
                sh.src[r + 1] = make_float4(P2P_FAR, P2P_FAR, 0.f, 0.f);
            }
            __syncthreads();
            // this warp's quarter of the source steps; the steps holding the
            // target leaf's own bodies need the r = 0 test
            const int nsteps = nsp / SPS;
            const int per = (nsteps + 3) >> 2;
            const int sb = warp * per, se = min(nsteps, sb + per);
            const int msteps = any_edge ? nsteps : max(0, (min(nself, s0 + ns) - s0 + SPS - 1) / SPS);
            // targets [t0, t0 + ntc) lie in window 0 as the leaf's own bodies
            const float* tsm = s0 == 0 && t0 + ntc <= ns ? srcf + 8 * (t0 >> 1) : nullptr;
            for (int c0 = 0; c0 < ntc; c0 += KM * LT) {
                const int rem = ntc - c0;
                if (KM >= 4 && rem > 3 * LT) p2p_cluster<(KM >= 4 ? 4 : 3), LT>(sh.src, tgt, tsm, c0, ntc, sb, se, msteps, lane, sh.part[warp]);
                else if (rem > 2 * LT) p2p_cluster<3, LT>(sh.src, tgt, tsm, c0, ntc, sb, se, msteps, lane, sh.part[warp]);
                else if (rem > LT) p2p_cluster<2, LT>(sh.src, tgt, tsm, c0, ntc, sb, se, msteps, lane, sh.part[warp]);
                else p2p_cluster<1, LT>(sh.src, tgt, tsm, c0, ntc, sb, se, msteps, lane, sh.part[warp]);
            }
        }
        __syncthreads();
        for (int i = tid; i < ntc; i += P2P_THREADS) {
            float4 r = sh.part[0][i];
            for (int w = 1; w < 4; w++) {
                r.x += sh.part[w][i].x;
                r.y += sh.part[w][i].y;
                r.z += sh.part[w][i].z;
                r.w += sh.part[w][i].w;
            }
            a.field[tb + t0 + i] = r;
        }
        __syncthreads();
    }
}

// One CTA per target leaf.
template <int LT, int KM = 3>
__global__ void __launch_bounds__(P2P_THREADS) k_p2p(const P2PArgs a)
{
    __shared__ P2PShared sh;
    p2p_init(sh);
    uint32_t phase = 0;
    p2p_leaf<LT, KM>(a, blockIdx.x, sh, phase);
}

// Persistent form: a fixed number of CTAs per SM walk the queue of leaves
// through an atomic counter (zero when the step starts), fetching the next leaf
// while they work on the current one.  With fewer CTAs than the SM holds, the
// concurrently running far-field kernels keep room to start.
template <int LT>
__global__ void __launch_bounds__(P2P_THREADS) k_p2p_queue(const P2PArgs a, int* counter, int nitems)
{
    __shared__ P2PShared sh;
    __shared__ int next;
    p2p_init(sh);
    uint32_t phase = 0;
    if (threadIdx.x == 0) next = atomicAdd(counter, 1);
    __syncthreads();
    int item = next;
    while (item < nitems) {
        __syncthreads();  // every thread has read 'next'
        if (threadIdx.x == 0) next = atomicAdd(counter, 1);
        p2p_leaf<LT>(a, (uint32_t)item, sh, phase);
        __syncthreads();
        item = next;
    }
}

// Batched form: the leaves of many systems in one queue.  Item i belongs to the
// system s with first[s] <= i < first[s+1] (systems ordered by work per leaf,
// heaviest first, so that the queue ends with the light leaves).
template <int LT, int KM = 3>
__global__ void __launch_bounds__(P2P_THREADS) k_p2p_batch(const P2PBatchArgs b)
{
    __shared__ P2PShared sh;
    __shared__ int next, leaf;
    __shared__ P2PArgs cur;
    p2p_init(sh);
    uint32_t phase = 0;
    if (threadIdx.x == 0) next = atomicAdd(b.counter, 1);
    __syncthreads();
    int item = next;
    while (item < b.nitems) {
        __syncthreads();  // every thread has read 'next' and finished with 'cur'
        if (threadIdx.x == 0) {
            next = atomicAdd(b.counter, 1);
            int lo = 0, hi = b.nsys - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (b.first[mid] <= item) lo = mid;
                else hi = mid - 1;
            }
            cur = b.sys[lo];
            leaf = item - b.first[lo];
        }
        __syncthreads();
        p2p_leaf<LT, KM>(cur, (uint32_t)leaf, sh, phase);
        __syncthreads();
        item = next;
    }
}

// Grid form of the batched near field: one CTA per queue item (no resident
// CTAs), so that the block scheduler interleaves the near field with the far-
// field kernels as CTAs retire (the far fields' stream priority then decides).
template <int LT, int KM = 3>
__global__ void __launch_bounds__(P2P_THREADS) k_p2p_batch_grid(const P2PBatchArgs b)
{
    __shared__ P2PShared sh;
    p2p_init(sh);
    uint32_t phase = 0;
    const int item = (int)blockIdx.x;
    int lo = 0, hi = b.nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&b.first[mid]) <= item) lo = mid;
        else hi = mid - 1;
    }
    p2p_leaf<LT, KM>(b.sys[lo], (uint32_t)(item - __ldg(&b.first[lo])), sh, phase);
}

int p2p_batch_shapes() { return 5; }

void launch_p2p_batch(const P2PBatchArgs& b, int shape, int per_sm, cudaStream_t s)
{
    if (b.nitems <= 0) return;
    COUNT_LAUNCH();
    if (per_sm <= 0) {
        const int grid = b.nitems;
        if (shape == 1) k_p2p_batch_grid<4><<<grid, P2P_THREADS, 0, s>>>(b);
        else if (shape == 2) k_p2p_batch_grid<16><<<grid, P2P_THREADS, 0, s>>>(b);
        else if (shape == 3) k_p2p_batch_grid<8, 4><<<grid, P2P_THREADS, 0, s>>>(b);
        else if (shape == 4) k_p2p_batch_grid<4, 4><<<grid, P2P_THREADS, 0, s>>>(b);
        else k_p2p_batch_grid<8><<<grid, P2P_THREADS, 0, s>>>(b);
        return;
    }
    const int grid = std::min(b.nitems, sm_count() * std::min(per_sm, 5));
    if (shape == 1) k_p2p_batch<4><<<grid, P2P_THREADS, 0, s>>>(b);
    else if (shape == 2) k_p2p_batch<16><<<grid, P2P_THREADS, 0, s>>>(b);
    else if (shape == 3) k_p2p_batch<8, 4><<<grid, P2P_THREADS, 0, s>>>(b);
    else if (shape == 4) k_p2p_batch<4, 4><<<grid, P2P_THREADS, 0, s>>>(b);
    else k_p2p_batch<8><<<grid, P2P_THREADS, 0, s>>>(b);
}

int p2p_variants() { return 3 * 5 + 2; }

void launch_p2p(const P2PArgs& a, int variant, cudaStream_t s, int* counter)
{
    const int nleaf = a.nleaf;
    COUNT_LAUNCH();
    if (variant >= 15) {  // one CTA per leaf, up to 4 targets per thread
        if (variant == 15) k_p2p<8, 4><<<nleaf, P2P_THREADS, 0, s>>>(a);
        else k_p2p<4, 4><<<nleaf, P2P_THREADS, 0, s>>>(a);
        return;
    }
    const int shape = variant % 3, per_sm = variant / 3;  // per_sm 0: one CTA per leaf
    if (per_sm == 0 || !counter) {
        if (shape == 1) k_p2p<4><<<nleaf, P2P_THREADS, 0, s>>>(a);
        else if (shape == 2) k_p2p<16><<<nleaf, P2P_THREADS, 0, s>>>(a);
        else k_p2p<8><<<nleaf, P2P_THREADS, 0, s>>>(a);
        return;
    }
    const int grid = std::min(nleaf, sm_count() * (per_sm + 1));  // 2..5 CTAs per SM
    if (shape == 1) k_p2p_queue<4><<<grid, P2P_THREADS, 0, s>>>(a, counter, nleaf);
    else if (shape == 2) k_p2p_queue<16><<<grid, P2P_THREADS, 0, s>>>(a, counter, nleaf);
    else k_p2p_queue<8><<<grid, P2P_THREADS, 0, s>>>(a, counter, nleaf);
}

// ------------------------------------------------------------------ M2M and L2L (one level per launch)

// Scaled M2M and L2L operators are the same at every level (cell size of the
// target level = 1): 8 dense R x R FP32 matrices, one per child octant, stored
// transposed ([octant][column][row]) so that a warp, 32 consecutive output rows,
// reads one line per column.  CTA = (32 rows) x (8 octants) of one parent cell:
// every thread runs a short chain (one octant, at most R columns) and the work of
// a level spreads over parents x ceil(R/32) CTAs.  Degree structure: an M2M output
// row of degree j reads inputs of degree <= j, an L2L output row of degree j
// inputs of degree >= j (kernel.cu:310-354, :408-454); both loops skip the zero
// blocks.


// M2M: M~_parent[r] = sum_oct sum_{c < (deg r + 1)^2} A_oct[r][c] M~_child(oct)[c];
// the 8 children of a parent are Morton-consecutive.  The octant sum is taken in
// octant order (deterministic).  grid = (nparent, ceil(R/32)), block = (32, 8).
__device__ __forceinline__ void m2m_body(const M2MArgs& ma, const int p, const int rb)
{
    extern __shared__ float ms[];  // the 8 children, 8 x R
    __shared__ float red[8][32];
    const float* __restrict__ Mc = ma.Mc;
    float* __restrict__ Mp = ma.Mp;
    const float* __restrict__ At = ma.At;
    const int R = ma.R, Rpad = ma.Rpad;
    const int o = threadIdx.y, r = rb * 32 + threadIdx.x;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    pdl_wait();
    pdl_trigger();
    for (int i = tid; i < 8 * R; i += 256) {
        const int oo = i / R;
        ms[i] = Mc[(size_t)(8 * p + oo) * Rpad + (i - oo * R)];
    }
    __syncthreads();
    float acc = 0.f;
    if (r < R) {
        const int j = real_degree(r), cend = (j + 1) * (j + 1);
        const float* a = At + (size_t)o * R * R + r;
        const float* m = ms + o * R;
#pragma unroll 4
        for (int c = 0; c < cend; c++) acc = fmaf(a[(size_t)c * R], m[c], acc);
    }
    red[o][threadIdx.x] = acc;
    __syncthreads();
    if (o == 0 && r < R) {
        float t = red[0][threadIdx.x];
#pragma unroll
        for (int k = 1; k < 8; k++) t += red[k][threadIdx.x];
        Mp[(size_t)p * Rpad + r] = t;
    }
}

__global__ void __launch_bounds__(256) k_m2m(const M2MArgs a) { m2m_body(a, blockIdx.x, blockIdx.y); }

void launch_m2m(const float* M_child, float* M_parent, const float* At, int nparent, int R, int Rpad, cudaStream_t s,
                bool pdl)
{
    COUNT_LAUNCH();
    M2MArgs a{M_child, M_parent, At, nparent, R, Rpad};
    launch_k(k_m2m, dim3(nparent, (R + 31) / 32), dim3(32, 8), sizeof(float) * 8 * R, s, pdl, a);
}

// P2M of 8 sibling leaves (one warp each, the arithmetic of k_p2m) followed by
// the M2M of their parent in the same CTA (the arithmetic of k_m2m: one thread
// per (octant, row), the octant sum in octant order), so that the leaf level
// and the level above it come out of one launch.  grid = nleaf / 8, block = 256.
template <int P>
__device__ __forceinline__ void p2m_m2m_body(const P2MArgs& pa, const int bid)
{
    constexpr int R = (P + 1) * (P + 1);
    constexpr int LD = 33;
    extern __shared__ float sm[];
    const int* off = pa.off;
    const float4* atoms = pa.atoms;
    float* M = pa.M;
    float* Mp = pa.Mp;
    const float* __restrict__ At = pa.At;
    const int Rpad = pa.Rpad;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int leaf = bid * 8 + warp;
    float* S = sm + warp * R * LD;
    float* ch = sm + 8 * R * LD;  // the 8 leaf multipoles
    float* red = ch + 8 * R;      // per-octant partial sums of the parent
    pdl_wait();
    pdl_trigger();
    for (int r = 0; r < R; r++) S[r * LD + lane] = 0.f;
    const int b = off[leaf], n = off[leaf + 1] - b;
    for (int c0 = 0; c0 < n; c0 += 32) {
        float4 a = c0 + lane < n ? atoms[b + c0 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float q = a.w;
        stream_regular<P>(a.x, a.y, a.z, [&](int nn, int mm, float yr, float yi) {
            float* sre = &S[ridx_re(nn, mm) * LD + lane];
            *sre = fmaf(q, yr, *sre);
            if (mm > 0) {
                float* sim = &S[ridx_im(nn, mm) * LD + lane];
                *sim = fmaf(-q, yi, *sim);
            }
        });
    }
    __syncwarp();
    float* out = M + (long)leaf * Rpad;
    for (int r = lane; r < R; r += 32) {
        float t = 0.f;
#pragma unroll 8
        for (int c = 0; c < 32; c++) t += S[r * LD + c];
        out[r] = t;
        ch[warp * R + r] = t;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * R; i += 256) {
        const int o = i / R, r = i - o * R;
        const int j = real_degree(r), cend = (j + 1) * (j + 1);
        const float* a = At + (size_t)o * R * R + r;
        const float* m = ch + o * R;
        float acc = 0.f;
#pragma unroll 4
        for (int c = 0; c < cend; c++) acc = fmaf(a[(size_t)c * R], m[c], acc);
        red[i] = acc;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < R; r += 256) {
        float t = red[r];
#pragma unroll
        for (int k = 1; k < 8; k++) t += red[k * R + r];
        Mp[(size_t)bid * Rpad + r] = t;
    }
}

template <int P>
__global__ void __launch_bounds__(256) k_p2m_m2m(const P2MArgs a) { p2m_m2m_body<P>(a, blockIdx.x); }

// Fused only while a CTA's shared memory allows several CTAs per SM (orders up
// to 7): at higher orders the standalone P2M keeps more warps resident.
constexpr size_t P2M_M2M_MAX_SMEM = 80 * 1024;

template <int P>
static bool p2m_m2m_dispatch(const int* off, int nleaf, const float4* atoms, float* M, float* Mp, const float* At,
                             int Rpad, cudaStream_t s, bool pdl)
{
    constexpr int R = (P + 1) * (P + 1);
    const size_t shm = sizeof(float) * (8 * R * 33 + 16 * R);
    if (shm > P2M_M2M_MAX_SMEM || nleaf % 8 != 0) return false;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_p2m_m2m<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        attr = true;
    }
    COUNT_LAUNCH();
    P2MArgs a{off, nleaf, atoms, M, Mp, At, Rpad};
    launch_k(k_p2m_m2m<P>, dim3(nleaf / 8), dim3(256), shm, s, pdl, a);
    return true;
}

bool launch_p2m_m2m(int P, const int* offsets, int nleaf, const float4* atoms, float* M_leaf, float* M_parent,
                    const float* At, int Rpad, cudaStream_t s, bool pdl)
{
    bool ok = false;
    GBFMM_ORDER_SWITCH(P, ok = p2m_m2m_dispatch<PP>(offsets, nleaf, atoms, M_leaf, M_parent, At, Rpad, s, pdl));
    return ok;
}


// ------------------------------------------------------------------ batched contraction (M2M, M2L, L2L)

// A CTA owns CT_TILE targets that share one operator per entry.  For each entry it
// gathers the source rows (transposed, [row][target]) into shared memory and runs
// a block-sparse FP32 GEMM: warps own (8-row block, column range) work items, the
// operator (packed [col][8 rows]) is read as broadcast float4 loads, each lane
// accumulates 8 rows x 2 targets.  Partial sums go to a shared [row][target] tile
// that is written (or added) to the destination level at the end.
__global__ void __launch_bounds__(CT_WARPS * 32) k_contract(ContractArgs a)
{
    extern __shared__ float sm[];
    const int R = a.R, Rpad = a.Rpad;
    constexpr int T = CT_TILE;
    constexpr int LT = CT_TILE + 1;
    float* Ms = sm;                       // R x T
    float* Ls = Ms + R * T;               // R x LT
    int* srow = reinterpret_cast<int*>(Ls + R * LT);
    int* trow = srow + T;
    const CTask task = a.tasks[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < R * LT; i += blockDim.x) Ls[i] = 0.f;
    int vt[3] = {0, 0, 0}, va[3] = {0, 0, 0};
    uint32_t tcode = 0;
    const bool tvalid = tid < task.ntgt;
    if (tid < T) {
        if (task.octant >= 0) {
            uint32_t q = (uint32_t)(task.q0 + tid);
            tcode = (q << 3) | (uint32_t)task.octant;
            morton_decode(q, va[0], va[1], va[2]);
        } else {
            tcode = (uint32_t)(task.q0 + tid);
        }
        morton_decode(tcode, vt[0], vt[1], vt[2]);
        trow[tid] = tvalid ? (int)(tcode * (uint32_t)Rpad) : -1;
    }
    // a tile whose targets hold no bodies (vacuum) needs no locals
    if (a.leaf_off) {
        bool occupied = false;
        if (tid < T && tvalid) {
            const int sh = 3 * (a.depth - task.level);
            occupied = a.leaf_off[(tcode + 1) << sh] > a.leaf_off[tcode << sh];
        }
        if (!__syncthreads_or(occupied)) return;
    }
    // this warp's work items (row block, column range) and their accumulators,
    // kept in registers across all entries of the task
    const int ib = a.warp_begin[task.group * (CT_WARPS + 1) + warp];
    const int nit = min(CT_MAXI, a.warp_begin[task.group * (CT_WARPS + 1) + warp + 1] - ib);
    int4 itm[CT_MAXI];
    int bofs[CT_MAXI];
    float acc[CT_MAXI][8][2];
#pragma unroll
    for (int k = 0; k < CT_MAXI; k++) {
        itm[k] = k < nit ? a.items[ib + k] : make_int4(0, 0, 0, 0);
        const BlockInfo bi = a.blocks[itm[k].x];
        bofs[k] = bi.off + (itm[k].y - bi.c0) * 8;
#pragma unroll
        for (int i = 0; i < 8; i++) acc[k][i][0] = acc[k][i][1] = 0.f;
    }
    for (int e = task.e_begin; e < task.e_end; e++) {
        const CEntry en = a.entries[e];
        const int slev = en.mode == 0 ? task.level : (en.mode == 1 ? task.level - 1 : task.level + 1);
        __syncthreads();
        if (tid < T) {
            int row = -1;
            if (tvalid) {
                if (en.mode == 2) {
                    row = (int)(((tcode << 3) | (uint32_t)((en.dx << 2) | (en.dy << 1) | en.dz)) * (uint32_t)Rpad);
                } else {
                    const int* base = en.mode == 0 ? vt : va;
                    int sx = base[0] + en.dx, sy = base[1] + en.dy, sz = base[2] + en.dz;
                    const int nx = grid_n(slev, a.shift[0]), ny = grid_n(slev, a.shift[1]),
                              nz = grid_n(slev, a.shift[2]);
                    bool ok = true;
                    if (a.periodic) {
                        sx &= nx - 1; sy &= ny - 1; sz &= nz - 1;
                    } else {
                        ok = sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz;
                    }
                    if (ok) row = (int)(morton_encode(sx, sy, sz) * (uint32_t)Rpad);
                }
            }
            srow[tid] = row;
        }
        __syncthreads();
        const float* src = a.src_lvl[slev];
        const int nc4 = Rpad >> 2;
        for (int idx = tid; idx < T * nc4; idx += blockDim.x) {
            const int t = idx % T, c4 = idx / T;
            const int row = srow[t];
            float4 v = row >= 0 ? __ldg(reinterpret_cast<const float4*>(src + row) + c4) : make_float4(0.f, 0.f, 0.f, 0.f);
            const int c = 4 * c4;
            if (c < R) Ms[c * T + t] = v.x;
            if (c + 1 < R) Ms[(c + 1) * T + t] = v.y;
            if (c + 2 < R) Ms[(c + 2) * T + t] = v.z;
            if (c + 3 < R) Ms[(c + 3) * T + t] = v.w;
        }
        __syncthreads();
        const float* op = a.ops + en.op;
#pragma unroll
        for (int k = 0; k < CT_MAXI; k++) {
            if (k < nit) {
                const float4* ap = reinterpret_cast<const float4*>(op + bofs[k]);
                for (int c = itm[k].y; c < itm[k].z; c++, ap += 2) {
                    const float4 a0 = __ldg(ap), a1 = __ldg(ap + 1);
                    const float2 m = *reinterpret_cast<const float2*>(&Ms[c * T + 2 * lane]);
                    acc[k][0][0] += a0.x * m.x; acc[k][0][1] += a0.x * m.y;
                    acc[k][1][0] += a0.y * m.x; acc[k][1][1] += a0.y * m.y;
                    acc[k][2][0] += a0.z * m.x; acc[k][2][1] += a0.z * m.y;
                    acc[k][3][0] += a0.w * m.x; acc[k][3][1] += a0.w * m.y;
                    acc[k][4][0] += a1.x * m.x; acc[k][4][1] += a1.x * m.y;
                    acc[k][5][0] += a1.y * m.x; acc[k][5][1] += a1.y * m.y;
                    acc[k][6][0] += a1.z * m.x; acc[k][6][1] += a1.z * m.y;
                    acc[k][7][0] += a1.w * m.x; acc[k][7][1] += a1.w * m.y;
                }
            }
        }
    }
    // fixed-order reduction of the warps' partial sums (pieces of one row block
    // may sit in different warps): warp 0 adds first, warp 7 last
    for (int w = 0; w < CT_WARPS; w++) {
        __syncthreads();
        if (warp == w) {
#pragma unroll
            for (int k = 0; k < CT_MAXI; k++) {
                if (k < nit) {
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const int r = 8 * itm[k].x + i;
                        if (r < R) {
                            Ls[r * LT + 2 * lane] += acc[k][i][0];
                            Ls[r * LT + 2 * lane + 1] += acc[k][i][1];
                        }
                    }
                }
            }
        }
    }
    __syncthreads();
    float* dst = a.dst_lvl[task.level];
    const int nr = task.r1 - task.r0;
    for (int idx = tid; idx < nr * T; idx += blockDim.x) {
        const int r = task.r0 + idx % nr, t = idx / nr;
        const int row = trow[t];
        if (row < 0) continue;
        const float v = Ls[r * LT + t];
        if (a.write_mode == 0) dst[row + r] = v;
        else if (a.write_mode == 1) dst[row + r] += v;
        else atomicAdd(&dst[row + r], v);
    }
}

void launch_contract(const ContractArgs& a, int ntasks, cudaStream_t s)
{
    if (ntasks <= 0) return;
    size_t shm = sizeof(float) * ((size_t)a.R * CT_TILE + (size_t)a.R * (CT_TILE + 1)) + sizeof(int) * 2 * CT_TILE;
    static size_t attr = 0;
    if (shm > attr) {
        cudaFuncSetAttribute(k_contract, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        attr = shm;
    }
    COUNT_LAUNCH();
    k_contract<<<ntasks, CT_WARPS * 32, shm, s>>>(a);
}

// ------------------------------------------------------------------ root (FP64)

// L~_0 = A_lattice M~_0 (images >= 2), and the FP32 copy of M~_0.  One warp per
// output row; lanes split the FP64 dot product, reduced by a fixed butterfly.
__device__ __forceinline__ void root_lattice_body(const RootArgs& a, const int bid)
{
    const int lane = threadIdx.x & 31;
    const int r = bid * 8 + (threadIdx.x >> 5);
    if (r >= a.R) return;
    double t = 0;
    if (a.images >= 2) {
        const double* A = a.lattice + (size_t)r * a.R;
        for (int c = lane; c < a.R; c += 32) t += A[c] * a.M0[c];
    }
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) {
        a.L0[r] = t;
        a.M0f[r] = (float)a.M0[r];
    }
}

__global__ void __launch_bounds__(256) k_root_lattice(const RootArgs a) { root_lattice_body(a, blockIdx.x); }

// L~_1[o] += A_o L~_0 (FP64 arithmetic, FP32 result).  One warp per (child, row).
__global__ void __launch_bounds__(256) k_root_l2l(RootArgs a)
{
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int o = w / a.R, r = w % a.R;
    if (o >= a.n1) return;
    const double* A = a.l2l + ((size_t)o * a.R + r) * a.R;
    double t = 0;
    for (int c = lane; c < a.R; c += 32) t += A[c] * a.L0[c];
    for (int k = 16; k > 0; k >>= 1) t += __shfl_xor_sync(0xffffffffu, t, k);
    if (lane == 0) a.L1[(size_t)o * a.Rpad + r] += (float)t;
}

void launch_root_lattice(const RootArgs& a, cudaStream_t s)
{
    COUNT_LAUNCH();
    k_root_lattice<<<(a.R + 7) / 8, 256, 0, s>>>(a);
}
void launch_root_l2l(const RootArgs& a, cudaStream_t s)
{
    COUNT_LAUNCH();
    k_root_l2l<<<(a.n1 * a.R + 7) / 8, 256, 0, s>>>(a);
}

// ------------------------------------------------------------------ upper tree in one launch

constexpr int TOP_THREADS = 512;

__host__ __device__ __forceinline__ bool top_staged(int R) { return R <= TOP_STAGE_MAX_R; }
__host__ __device__ __forceinline__ int top_r2p(int R) { return (R * R + 1) & ~1; }  // FP64 block stride

// Shared memory of k_top.  Staged: FP32 M2M operator (8 R^2) | FP64 root M2M
// block of the CTA's octant (R2p) | FP64 lattice (R2p) | input cells (64 rows of
// Rpad) | M~_0 (R, FP64) | level 1 as FP64 (R) | level 1 (Rpad) | level 2
// (8 Rpad) | octant partials (64 R).  Unstaged: M~_0, level 1 (FP64, FP32).
size_t top_smem_bytes(int R)
{
    const size_t r = (size_t)R, rp = (size_t)((R + 3) & ~3), r2p = (size_t)top_r2p(R);
    if (!top_staged(R)) return sizeof(double) * 2 * r + sizeof(float) * rp;
    return sizeof(float) * 8 * r * r + sizeof(double) * (2 * r2p + 2 * r) + sizeof(float) * (73 * rp + 64 * r);
}

// M2M of np parents whose 8 children sit in ch[(8p + o) Rpad + c], operator At
// [octant][column][row], all in shared memory.  A thread owns (octant, row) of
// up to four parents: one operator read feeds four independent chains.  Each
// (parent, octant, row) sum runs over the columns in order and the octant sum is
// taken in octant order: the arithmetic of k_m2m.  Parents go to par (shared,
// stride Rpad) and dst (global, stride Rpad).
__device__ __forceinline__ void top_m2m(const float* ch, float* red, float* par, float* dst, int np, const float* At,
                                        int R, int Rpad)
{
    const int pq = np >= 4 ? 4 : 1, ng = np / pq;
    for (int i = threadIdx.x; i < ng * 8 * R; i += TOP_THREADS) {
        const int r = i % R, o = (i / R) & 7, p0 = (i / (8 * R)) * pq;
        const int j = real_degree(r), cend = (j + 1) * (j + 1);
        const float* a = At + o * R * R + r;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        if (pq == 4) {
            const float* m0 = ch + (8 * p0 + o) * Rpad;
#pragma unroll 2
            for (int c = 0; c < cend; c++) {
                const float w = a[c * R];
#pragma unroll
                for (int k = 0; k < 4; k++) acc[k] = fmaf(w, m0[8 * k * Rpad + c], acc[k]);
            }
#pragma unroll
            for (int k = 0; k < 4; k++) red[(8 * (p0 + k) + o) * R + r] = acc[k];
        } else {
            const float* m0 = ch + (8 * p0 + o) * Rpad;
#pragma unroll 4
            for (int c = 0; c < cend; c++) acc[0] = fmaf(a[c * R], m0[c], acc[0]);
            red[(8 * p0 + o) * R + r] = acc[0];
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < np * R; i += TOP_THREADS) {
        const int p = i / R, r = i - p * R;
        float t = red[8 * p * R + r];
#pragma unroll
        for (int k = 1; k < 8; k++) t += red[(8 * p + k) * R + r];
        par[p * Rpad + r] = t;
        dst[(size_t)p * Rpad + r] = t;
    }
    __syncthreads();
}

// Fixed pairwise tree over the 4 x 8 shares of one root row ((octant, quarter)
// index k = 4 o + q): five dependent FP64 additions instead of 31 (an FP64 add
// waits ~64 cycles for its predecessor on GB300).
__device__ __forceinline__ double tree_sum32(double (&v)[32])
{
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1)
#pragma unroll
        for (int k = 0; k < w; k++) v[k] = v[k] + v[k + w];
    return v[0];
}

// CTA g owns the subtree of level-1 cell g.  Staged form (R <= TOP_STAGE_MAX_R):
// the operators and the input cells arrive by bulk copies on one mbarrier (one
// memory latency), then M2M from level 'from' (3 or 2) up to level 1 in shared
// memory.  Both forms then take the CTA's share of the FP64 root M2M
// M~_0 = sum_o A_o M~_1[o] (octant g; columns in four quarters, one thread per
// (row, quarter)); the last CTA to finish adds the 32 shares of a row by a fixed
// pairwise tree and applies the lattice operator (one thread per (row, column
// quarter), quarters added pairwise), so that the upper tree takes one launch.
// The degree-0 and degree-1 moments of M~_0 (total charge and dipole about the
// box centre) are replaced by sums over the bodies of exact products in FP32
// pairs (about 48 bits; the tree-key kernel's per-block partials, summed here),
// which is what the reference's FP64 P2M/M2M produces to that accuracy: the FP32
// upward pass would otherwise leave a monopole residual of ~1e-7 of sum|q| that
// the periodic lattice operator (about 81 periods wide) turns into a constant
// shift of every potential.
template <bool STAGED>
__device__ __forceinline__ void top_body(const TopArgs& a, const int bid, const int nb)
{
    extern __shared__ float4 topsm[];
    __shared__ uint64_t bar;
    static_assert(TOP_LATTICE_MAX_R <= 64, "lattice quarters buffer");
    __shared__ double lq[4 * 64];  // lattice quarters (R <= TOP_LATTICE_MAX_R rows)
    const int R = a.root.R, Rpad = a.root.Rpad, R2p = top_r2p(R), g = bid, tid = threadIdx.x;
    float* At = reinterpret_cast<float*>(topsm);
    double* Ag = reinterpret_cast<double*>(At + (STAGED ? 8 * R * R : 0));
    double* lat = Ag + (STAGED ? R2p : 0);
    float* in = reinterpret_cast<float*>(lat + (STAGED ? R2p : 0));
    double* M0s = reinterpret_cast<double*>(in + (STAGED ? 64 * Rpad : 0));
    double* m1d = M0s + R;
    float* m1 = reinterpret_cast<float*>(m1d + R);
    float* mid = m1 + Rpad;
    float* red = mid + 8 * Rpad;
    if (STAGED) {
        // bulk copies: 8 R^2 floats, R2p doubles and Rpad-float rows are all
        // multiples of 16 bytes; the sources are 16-byte aligned allocations
        const int rows = a.from == 3 ? 64 : a.from == 2 ? 8 : 1;
        const float* src_in = a.from >= 2 ? a.Min + (size_t)rows * g * Rpad : a.M1 + (size_t)g * Rpad;
        const uint32_t b_in = 4u * rows * Rpad;
        if (tid == 0) {
            // the operators are constant: their copies may start before the
            // previous kernel's end (pdl_wait), the input cells' after it
            mbar_init(&bar, 1);
            mbar_init_fence();
            const uint32_t b_at = a.from >= 2 ? 32u * R * R : 0u, b_ag = 8u * R2p, b_lat = a.lattice ? 8u * R2p : 0u;
            mbar_expect_tx(&bar, b_at + b_ag + b_lat + b_in);
            if (b_at) bulk_g2s(At, a.m2m_t, b_at, &bar);
            bulk_g2s(Ag, a.root.m2m + (size_t)g * R2p, b_ag, &bar);
            if (b_lat) bulk_g2s(lat, a.root.lattice, b_lat, &bar);
        }
        pdl_wait();
        if (tid == 0) bulk_g2s(a.from == 3 ? in : a.from == 2 ? mid : m1, src_in, b_in, &bar);
        __syncthreads();
        if (!mbar_wait(&bar, 0, a.err, 1, a.wait_limit))
            mbar_drain(&bar, 0, a.wait_limit);  // no exit while the copies may still land
        if (a.from == 3) top_m2m(in, red, mid, a.M2 + (size_t)8 * g * Rpad, 8, At, R, Rpad);
        if (a.from >= 2) top_m2m(mid, red, m1, a.M1 + (size_t)g * Rpad, 1, At, R, Rpad);
    } else {
        pdl_wait();
        for (int r = tid; r < R; r += TOP_THREADS) m1[r] = a.M1[(size_t)g * Rpad + r];
        __syncthreads();
    }
    for (int r = tid; r < R; r += TOP_THREADS) m1d[r] = (double)m1[r];
    __syncthreads();
    const int qc = (R + 3) / 4;
    // the root-M2M shares of every octant whose cell is this CTA's stored cell
    // (a slab's root cube repeats the box along x and y: octants g, g+2, g+4, g+6)
    for (int o = g; o < 8; o++) {
        if ((o & a.umask) != g) continue;
        const double* A0 = (STAGED && o == g) ? Ag : a.root.m2m + (size_t)o * R2p;
        for (int i = tid; i < 4 * R; i += TOP_THREADS) {
            const int r = i >> 2, p = i & 3;
            const double* A = A0 + (size_t)r * R;
            double t = 0;
            for (int c = p * qc; c < min(R, (p + 1) * qc); c++) t = fma(A[c], m1d[c], t);
            a.part[((size_t)o * R + r) * 4 + p] = t;
        }
    }
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(a.done, 1) == (int)nb - 1;
    __syncthreads();
    if (!s_last) return;
    pdl_trigger();  // the other CTAs have exited: the next kernel may launch
    __threadfence();
    if (tid == 0) *a.done = 0;  // ready for the next step
    // dipole (3) and total charge of the bodies: the tree-key kernel's per-block
    // partials, one warp per quantity
    __shared__ double sums[4];
    if (tid < 128) {
        const double t = sum_tree_partials(a.tree_part, a.tree_nblocks, tid >> 5);
        if ((tid & 31) == 0) {
            sums[tid >> 5] = t;
            a.sums[tid >> 5] = t;
        }
    }
    __syncthreads();
    for (int r = tid; r < R; r += TOP_THREADS) {
        double v[32];
#pragma unroll
        for (int k = 0; k < 32; k++) v[k] = __ldcg(&a.part[((size_t)(k >> 2) * R + r) * 4 + (k & 3)]);
        double s = tree_sum32(v);
        if (r < 4) {
            // the root cube holds 'copies' copies of the box, whose dipole about
            // the root centre is copies x (box dipole about the box centre)
            const StepConst* sc = a.root.sc;
            // (divisions by the root edge as products with its host-computed
            // reciprocal: an FP64 division is a long dependent chain here)
            const double Q = sums[3], iL = sc->inv_box_len, k = (double)sc->copies;
            if (r == 0) s = k * Q;
            else if (r == 1) s = -k * (sums[2] - Q * sc->box_centre[2]) * iL;
            else if (r == 2) s = k * (sums[0] - Q * sc->box_centre[0]) * (0.5 * iL);
            else s = -k * (sums[1] - Q * sc->box_centre[1]) * (0.5 * iL);
        }
        M0s[r] = s;
        a.root.M0[r] = s;
    }
    if (tid == 0) {
        // FP32 constants of the tin-foil dipole correction for the finalize
        // (solver.cpp:30-49): q * ke * coef * M per body and ke * coef * |M|^2 / N
        const double M0 = sums[0], M1 = sums[1], M2 = sums[2];
        const double cK = a.root.sc->coef * KE;
        a.fconst[0] = (float)(cK * M0);
        a.fconst[1] = (float)(cK * M1);
        a.fconst[2] = (float)(cK * M2);
        a.fconst[3] = (float)(cK * (M0 * M0 + M1 * M1 + M2 * M2) * a.inv_natoms);
    }
    __syncthreads();
    if (!a.lattice) return;
    const double* Alat = STAGED ? lat : a.root.lattice;
    for (int i = tid; i < 4 * R; i += TOP_THREADS) {
        const int r = i >> 2, p = i & 3;
        const double* A = Alat + (size_t)r * R;
        double t = 0;
        if (a.root.images >= 2)
            for (int c = p * qc; c < min(R, (p + 1) * qc); c++) t = fma(A[c], M0s[c], t);
        lq[i] = t;
    }
    __syncthreads();
    for (int r = tid; r < R; r += TOP_THREADS) {
        a.root.L0[r] = (lq[4 * r] + lq[4 * r + 1]) + (lq[4 * r + 2] + lq[4 * r + 3]);
        a.root.M0f[r] = (float)M0s[r];
    }
}

template <bool STAGED>
__global__ void __launch_bounds__(TOP_THREADS) k_top(const TopArgs a) { top_body<STAGED>(a, blockIdx.x, gridDim.x); }

void launch_top(const TopArgs& a, cudaStream_t s, bool pdl)
{
    const size_t shm = top_smem_bytes(a.root.R);
    const bool staged = top_staged(a.root.R);
    static size_t attr[2] = {0, 0};
    if (shm > attr[staged]) {
        if (staged) cudaFuncSetAttribute(k_top<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        else cudaFuncSetAttribute(k_top<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        attr[staged] = shm;
    }
    COUNT_LAUNCH();
    if (staged) launch_k(k_top<true>, dim3(a.root.n1), dim3(TOP_THREADS), shm, s, pdl, a);
    else launch_k(k_top<false>, dim3(a.root.n1), dim3(TOP_THREADS), shm, s, pdl, a);
    if (!a.lattice) launch_root_lattice(a.root, s);
}

// ------------------------------------------------------------------ bounded-wait probe

__global__ void k_wait_probe(uint32_t polls, int* err)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    // nothing arrives on the barrier: phase 0 never completes
    if (threadIdx.x == 0) mbar_wait(&bar, 0, err, 1, polls);
    __syncthreads();
}

void launch_wait_probe(uint32_t polls, int* err, cudaStream_t s)
{
    COUNT_LAUNCH();
    k_wait_probe<<<1, 32, 0, s>>>(polls, err);
}

// ------------------------------------------------------------------ finalize

// Unit conversion of gpu_solver.cu:250-256 (phi*ke, F = -q*ke*grad phi), the
// tin-foil dipole correction of solver.cpp:30-49, scatter back to input order
// (solver.cpp:58-67) and the FP64 energy 0.5*sum(q*phi) (fmm.cpp:89-98).
__device__ __forceinline__ void finalize_body(const FinalArgs& a, const int bid, const int nb)
{
    // FP32 constants of the dipole correction, computed once in FP64 by k_top
    const float fM0 = a.fconst[0], fM1 = a.fconst[1], fM2 = a.fconst[2], corr_f = a.fconst[3];
    const float inv_h = a.sc->inv_h, inv_h2 = a.sc->inv_h * a.sc->inv_h;
    float* __restrict__ forces = a.sc->out_forces;
    float* __restrict__ pots = a.sc->out_pots;
    f2sum e = {0.f, 0.f};
    // in input order (coalesced writes, to device or host memory), gathering
    // each body's fields from its sorted position
    for (int o = bid * blockDim.x + threadIdx.x; o < a.n; o += nb * blockDim.x) {
        const int i = a.inv[o];
        const float4 nf = a.near[i], ff = a.far[i];
        const float q = a.atoms[i].w;
        const float phi = (nf.x + ff.x) * inv_h;
        const float gx = (nf.y + ff.y) * inv_h2, gy = (nf.z + ff.z) * inv_h2, gz = (nf.w + ff.w) * inv_h2;
        const float qk = -q * (float)KE;
        forces[3 * o] = qk * gx + q * fM0;
        forces[3 * o + 1] = qk * gy + q * fM1;
        forces[3 * o + 2] = qk * gz + q * fM2;
        // FP32 per body (no FP64 division); the exact products of the energy are
        // summed as FP32 pairs, per block and then over the blocks
        float pot = phi * (float)KE;
        if (q != 0.f) pot -= corr_f / q;
        pots[o] = pot;
        e = f2s_add(e, f2s_prod(0.5f * q, pot));  // the exact product, as FP64 would hold it
    }
    e = f2s_warp_sum(e);
    __shared__ f2sum red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        f2sum t = red[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) t = f2s_add(t, red[w]);
        reinterpret_cast<f2sum*>(a.partials)[bid] = t;
    }
    if (!a.done) return;
    // last block: the energy, partials summed in a fixed order
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(a.done, 1) == (int)nb - 1;
    __syncthreads();
    if (!s_last || threadIdx.x >= 32) return;
    __threadfence();
    if (threadIdx.x == 0) {
        // ready for the next step: this counter and the one after the near field
        *a.done = 0;
        if (a.zero_after) *a.zero_after = 0;
    }
    // the energy: the blocks' FP32-pair partials summed in FP32 pairs (sum_partials)
    const double t = sum_partials(reinterpret_cast<const float2*>(a.partials), 1, (int)nb);
    if (threadIdx.x == 0) {
        *a.sc->out_energy = t;
        int* fl = a.sc->out_flags;
        if (fl)
            for (int k = 0; k < 4; k++) fl[k] = __ldcg(&a.flags[k]);
    }
}

__global__ void __launch_bounds__(256) k_finalize(const FinalArgs a) { finalize_body(a, blockIdx.x, gridDim.x); }

void launch_finalize(const FinalArgs& a, cudaStream_t s)
{
    int blocks = final_blocks(a.n);
    COUNT_LAUNCH();
    k_finalize<<<blocks, 256, 0, s>>>(a);
}

}  // namespace gbfmm

namespace gbfmm {

// ------------------------------------------------------------------ batched launches
//
// One launch runs a kernel for many systems: CTA b runs block b - first[s] of
// system s, where first[] (device) holds the prefix sums of the systems' grid
// sizes; each system's arguments are a struct in device memory.  The bodies are
// those of the single-system kernels, so every system's arithmetic is the same.

__device__ __forceinline__ int batch_system(const int* first, int nsys, int b)
{
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&first[mid]) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

#define GBFMM_BATCH_PROLOGUE                                     \
    const int sys = batch_system(first, nsys, (int)blockIdx.x); \
    const int b0 = __ldg(&first[sys]), nb = __ldg(&first[sys + 1]) - b0, bid = (int)blockIdx.x - b0;

__global__ void __launch_bounds__(256) k_tree_keys_batch(const TreeArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    tree_keys_body(as[sys], bid, nb);
}

__global__ void k_scatter_ranked_batch(const ScatterArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    (void)nb;
    scatter_ranked_body(as[sys], bid);
}

__global__ void __launch_bounds__(256) k_leaf_sort_batch(const LeafSortArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    (void)nb;
    leaf_sort_body(as[sys], bid);
}

template <int P, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_p2m_batch(const P2MArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    (void)nb;
    p2m_body<P, WARPS>(as[sys], bid);
}

template <int P>
__global__ void __launch_bounds__(256) k_p2m_m2m_batch(const P2MArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    (void)nb;
    p2m_m2m_body<P>(as[sys], bid);
}

template <int P, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_l2p_batch(const L2PArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    (void)nb;
    l2p_body<P, WARPS>(as[sys], bid);
}

template <int P>
__global__ void __launch_bounds__(256) k_down_batch(const DownArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    (void)nb;
    down_body<P>(as[sys], bid);
}

// M2M: system s's block lb is (parent lb / row blocks, row block lb % row blocks).
__global__ void __launch_bounds__(256) k_m2m_batch(const M2MArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    (void)nb;
    const M2MArgs& a = as[sys];
    const int nrb = (a.R + 31) / 32;
    m2m_body(a, bid / nrb, bid % nrb);
}

template <bool STAGED>
__global__ void __launch_bounds__(TOP_THREADS) k_top_batch(const TopArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    top_body<STAGED>(as[sys], bid, nb);
}

__global__ void __launch_bounds__(256) k_root_lattice_batch(const RootArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    (void)nb;
    root_lattice_body(as[sys], bid);
}

__global__ void __launch_bounds__(256) k_finalize_batch(const FinalArgs* as, const int* first, int nsys)
{
    GBFMM_BATCH_PROLOGUE
    finalize_body(as[sys], bid, nb);
}

template <int P>
static void launch_p2m_batch_t(const P2MArgs* args, const int* first, int nsys, int nblocks, size_t smem,
                               cudaStream_t s)
{
    constexpr int R = (P + 1) * (P + 1);
    constexpr int W = R <= 169 ? 4 : 2;
    static size_t attr = 0;
    if (smem > attr) {
        cudaFuncSetAttribute(k_p2m_batch<P, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = smem;
    }
    k_p2m_batch<P, W><<<nblocks, W * 32, smem, s>>>(args, first, nsys);
}

template <int P>
static void launch_down_batch_t(const DownArgs* args, const int* first, int nsys, int nblocks, cudaStream_t s)
{
    const size_t shm = down_smem_bytes(P);
    static bool attr = false;
    if (!attr && shm > 0) {
        cudaFuncSetAttribute(k_down_batch<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        attr = true;
    }
    k_down_batch<P><<<nblocks, 256, shm, s>>>(args, first, nsys);
}

template <int P>
static void launch_p2m_m2m_batch_t(const P2MArgs* args, const int* first, int nsys, int nblocks, size_t smem,
                                   cudaStream_t s)
{
    static size_t attr = 0;
    if (smem > attr) {
        cudaFuncSetAttribute(k_p2m_m2m_batch<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = smem;
    }
    k_p2m_m2m_batch<P><<<nblocks, 256, smem, s>>>(args, first, nsys);
}

void launch_batch(BatchKernel k, int P, const void* args, const int* first, int nsys, int nblocks, size_t smem,
                  cudaStream_t s)
{
    if (nsys <= 0 || nblocks <= 0) return;
    COUNT_LAUNCH();
    switch (k) {
        case BatchKernel::TREE_KEYS:
            k_tree_keys_batch<<<nblocks, 256, smem, s>>>((const TreeArgs*)args, first, nsys);
            break;
        case BatchKernel::SCATTER:
            k_scatter_ranked_batch<<<nblocks, 256, 0, s>>>((const ScatterArgs*)args, first, nsys);
            break;
        case BatchKernel::LEAF_SORT:
            k_leaf_sort_batch<<<nblocks, 256, 0, s>>>((const LeafSortArgs*)args, first, nsys);
            break;
        case BatchKernel::P2M:
            GBFMM_ORDER_SWITCH(P, launch_p2m_batch_t<PP>((const P2MArgs*)args, first, nsys, nblocks, smem, s));
            break;
        case BatchKernel::P2M_M2M:
            GBFMM_ORDER_SWITCH(P, launch_p2m_m2m_batch_t<PP>((const P2MArgs*)args, first, nsys, nblocks, smem, s));
            break;
        case BatchKernel::L2P:
            GBFMM_ORDER_SWITCH(P, (k_l2p_batch<PP, 4><<<nblocks, 128, 0, s>>>((const L2PArgs*)args, first, nsys)));
            break;
        case BatchKernel::DOWN:
            GBFMM_ORDER_SWITCH(P, launch_down_batch_t<PP>((const DownArgs*)args, first, nsys, nblocks, s));
            break;
        case BatchKernel::M2M:
            k_m2m_batch<<<nblocks, dim3(32, 8), smem, s>>>((const M2MArgs*)args, first, nsys);
            break;
        case BatchKernel::TOP_STAGED:
        case BatchKernel::TOP_UNSTAGED: {
            const bool staged = k == BatchKernel::TOP_STAGED;
            static size_t attr[2] = {0, 0};
            if (smem > attr[staged]) {
                if (staged) cudaFuncSetAttribute(k_top_batch<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                else cudaFuncSetAttribute(k_top_batch<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                attr[staged] = smem;
            }
            if (staged) k_top_batch<true><<<nblocks, TOP_THREADS, smem, s>>>((const TopArgs*)args, first, nsys);
            else k_top_batch<false><<<nblocks, TOP_THREADS, smem, s>>>((const TopArgs*)args, first, nsys);
            break;
        }
        case BatchKernel::ROOT_LATTICE:
            k_root_lattice_batch<<<nblocks, 256, 0, s>>>((const RootArgs*)args, first, nsys);
            break;
        case BatchKernel::FINALIZE:
            k_finalize_batch<<<nblocks, 256, 0, s>>>((const FinalArgs*)args, first, nsys);
            break;
        default:
            break;
    }
}

}  // namespace gbfmm

namespace gbfmm {

size_t p2m_smem_bytes(int P)
{
    const int R = (P + 1) * (P + 1);
    return sizeof(float) * (size_t)p2m_warps(P) * R * 33;
}

int p2m_warps(int P)
{
    const int R = (P + 1) * (P + 1);
    return R <= 169 ? 4 : 2;
}

size_t p2m_m2m_smem_bytes(int P)
{
    const int R = (P + 1) * (P + 1);
    const size_t shm = sizeof(float) * ((size_t)8 * R * 33 + 16 * R);
    return shm > P2M_M2M_MAX_SMEM ? 0 : shm;
}

}  // namespace gbfmm
