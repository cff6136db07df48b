// Coulomb virial of the last step: Xi = -1/2 sum_pairs r_ij (x) F_ij, with the
// pair sum over the same periodic images as the step's lattice sum.
//
// Writing r_ijn = r_i - r_j - n.L for the pair of body i and the image n of
// body j, and using f_ijn = -f_{j,i,-n} (a symmetric set of images):
//   sum_{i,j,n} r_ijn (x) f_ijn = 2 sum_i r_i (x) F_i - G,
//   G = sum_{i,j,n} (n.L) (x) f_ijn,
// so Xi_lattice = -1/2 sum_i r_i (x) F_i + G / 4, and the tin-foil correction
// (energy -(2 pi / 3V) |M|^2 ke) adds -(pi ke / 3V)(2 M (x) M - |M|^2 I).  G, the
// force of every interaction weighted by the period shift of its source image,
// is non-zero only where an interaction crosses the box: the near-field stencil
// entries and M2L stencil entries whose source cell wraps around the periodic
// grid, and the far lattice images of the root.  Each is computed from the
// step's own tree, expansions and operators:
//   k_vir_p2p   per target leaf, the body-body forces of the wrapped near-field
//               entries, weighted by their shift;
//   k_vir_m2l   per target cell, the M2L contributions of the wrapped entries
//               accumulated into three extra local expansions Lambda_a, each
//               weighted by the shift along axis a;
//   k_vir_root  the far lattice weighted by the image index (FP64, operators of
//               lattice_shift_operators) at the root, L2L to level 1;
//   then the step's downward pass (L2L and L2P) on each Lambda_a, and
//   k_vir_reduce sums r_i (x) F_i and the Lambda_a forces over the bodies.
// No counterpart in the reference: its plugin adds forces without a virial
// (zeta_fmm_solver.cpp:66-76), where mdrun's ForceWithVirial expects one
// (sim_util.cpp:2085).
#include <cuda_runtime.h>

#include <atomic>

#include "common.cuh"
#include "kernels.h"

namespace gbfmm {

extern std::atomic<long> g_kernel_launches;

namespace {

__device__ __forceinline__ int floordiv(int a, int n) { return a >= 0 ? a / n : -((-a + n - 1) / n); }

__device__ __forceinline__ float block_sum(float v, float* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    return t;
}

}  // namespace

// One CTA (128 threads) per target leaf: for each near-field stencil entry whose
// source leaf wraps around the box (shift n != 0), F = sum over the leaves'
// body pairs of q_i q_j (u_i - u_j - d) / |.|^3 (scaled units), and
// part[9 leaf + 3a + b] = sum n_a F_b.
__global__ void __launch_bounds__(128) k_vir_p2p(const P2PArgs a, double* part)
{
    __shared__ float red[3][4];
    const uint32_t t = blockIdx.x;
    int tx, ty, tz;
    morton_decode(t, tx, ty, tz);
    const int tb = a.off[t], nt = a.off[t + 1] - tb;
    double g[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (nt > 0 && a.periodic) {
        for (int e = 0; e < a.nst; e++) {
            const int dx = a.stencil[3 * e], dy = a.stencil[3 * e + 1], dz = a.stencil[3 * e + 2];
            const int wx = floordiv(tx + dx, a.nd[0]), wy = floordiv(ty + dy, a.nd[1]), wz = floordiv(tz + dz, a.nd[2]);
            if (wx == 0 && wy == 0 && wz == 0) continue;  // uniform over the CTA
            const uint32_t sc = morton_encode(tx + dx - wx * a.nd[0], ty + dy - wy * a.nd[1], tz + dz - wz * a.nd[2]);
            const int sb = a.off[sc], ns = a.off[sc + 1] - sb;
            float f[3] = {0.f, 0.f, 0.f};
            for (int p = threadIdx.x; p < nt * ns; p += blockDim.x) {
                const int i = p / ns, j = p - i * ns;
                const float4 bi = a.atoms[tb + i], bj = a.atoms[sb + j];
                const float ex = bi.x - (bj.x + (float)dx), ey = bi.y - (bj.y + (float)dy), ez = bi.z - (bj.z + (float)dz);
                const float r2 = ex * ex + ey * ey + ez * ez;
                if (r2 > 0.f) {
                    const float ri = rsqrtf(r2);
                    const float s = bi.w * bj.w * ri * ri * ri;
                    f[0] += s * ex;
                    f[1] += s * ey;
                    f[2] += s * ez;
                }
            }
            const int n[3] = {wx, wy, wz};
            for (int c = 0; c < 3; c++) {
                const float F = block_sum(f[c], red[c]);
                for (int r = 0; r < 3; r++) g[3 * r + c] += (double)n[r] * (double)F;
            }
        }
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 9; c++) part[9 * (size_t)t + c] = g[c];
}

// One warp per target cell of levels 1..D: for each M2L stencil entry whose
// source cell wraps (shift n != 0), y = T M~_src (dense transposed FP32 operator
// of the entry's class), and Lambda_a += n_a y.  Lambda_a rows are written, not
// added: one warp owns a cell.
__global__ void __launch_bounds__(256) k_vir_m2l(const VirialM2LArgs a)
{
    extern __shared__ float vsm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    long w = (long)blockIdx.x * 8 + wib;
    int k = 1;
    while (k <= a.depth && w >= a.ncell[k]) {
        w -= a.ncell[k];
        k++;
    }
    if (k > a.depth) return;
    const int R = a.R;
    float* msrc = vsm + wib * a.Rpad;
    const uint32_t c = (uint32_t)w, s = c & 7u, q = c >> 3;
    int vt[3], va[3];
    morton_decode(c, vt[0], vt[1], vt[2]);
    morton_decode(q, va[0], va[1], va[2]);
    const int lt = k == 1 ? 0 : 1;
    const int e0 = a.e_first[lt][s], ne = a.e_count[lt][s];
    constexpr int RPL = VIR_MAXR / 32;
    float acc[3][RPL];
#pragma unroll
    for (int x = 0; x < 3; x++)
#pragma unroll
        for (int r = 0; r < RPL; r++) acc[x][r] = 0.f;
    for (int e = 0; e < ne; e++) {
        const CEntry en = a.entries[e0 + e];
        const int slev = en.mode == 0 ? k : k - 1;
        const int* base = en.mode == 0 ? vt : va;
        int src[3] = {base[0] + en.dx, base[1] + en.dy, base[2] + en.dz}, n[3];
        for (int d = 0; d < 3; d++) {
            const int m = grid_n(slev, a.shift[d]);
            n[d] = floordiv(src[d], m);
            src[d] -= n[d] * m;
        }
        if (n[0] == 0 && n[1] == 0 && n[2] == 0) continue;  // uniform over the warp
        const float* M = a.M[slev] + (size_t)morton_encode(src[0], src[1], src[2]) * a.Rpad;
        __syncwarp();
        for (int r = lane; r < R; r += 32) msrc[r] = M[r];
        __syncwarp();
        const float* T = a.ops + (size_t)en.op * R * R;  // [column][row]
#pragma unroll
        for (int rr = 0; rr < RPL; rr++) {
            const int r = lane + 32 * rr;
            if (r < R) {
                float y = 0.f;
                for (int col = 0; col < R; col++) y = fmaf(T[(size_t)col * R + r], msrc[col], y);
#pragma unroll
                for (int x = 0; x < 3; x++) acc[x][rr] = fmaf((float)n[x], y, acc[x][rr]);
            }
        }
    }
#pragma unroll
    for (int rr = 0; rr < RPL; rr++) {
        const int r = lane + 32 * rr;
        if (r < R)
#pragma unroll
            for (int x = 0; x < 3; x++) a.lam[x][k][(size_t)c * a.Rpad + r] = acc[x][rr];
    }
}

// Block x = axis a: Lambda_a at the root = A_a M~_0 (FP64, the shift-weighted
// far lattice), then Lambda_a of the stored level-1 cells += L2L_o (Lambda_a root).
__global__ void __launch_bounds__(256) k_vir_root(const VirialRootArgs a)
{
    extern __shared__ double vroot[];
    const int x = blockIdx.x, R = a.R;
    double* L0 = vroot;
    const double* A = a.lat_shift + (size_t)x * R * R;
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        double t = 0;
        for (int col = 0; col < R; col++) t = fma(A[(size_t)r * R + col], a.M0[col], t);
        L0[r] = t * a.scale[x];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < a.n1 * R; i += blockDim.x) {
        const int o = i / R, r = i - o * R;
        const double* B = a.l2l + ((size_t)o * R + r) * R;
        double t = 0;
        for (int col = 0; col < R; col++) t = fma(B[col], L0[col], t);
        a.lam1[x][(size_t)o * a.Rpad + r] += (float)t;
    }
}

// Grid-stride over the leaves: per body r = leaf centre + u h, F = -q ke grad
// (near + far, without the tin-foil term), and the forces of the three shift
// expansions; per block the FP64 sums W[3a+b] = sum r_a F_b,
// Gf[3a+b] = sum F_b[Lambda_a] and Gp = sum of the near-field partials of its leaves.
__global__ void __launch_bounds__(256) k_vir_reduce(const VirialReduceArgs a)
{
    double w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, gf[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0},
           gp[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const StepConst* sc = a.sc;
    const float inv_h = sc->inv_h;
    const double h = 1.0 / (double)inv_h, kf = KE * (double)inv_h * (double)inv_h;
    for (int leaf = blockIdx.x; leaf < a.nleaf; leaf += gridDim.x) {
        if (threadIdx.x == 0)
            for (int c = 0; c < 9; c++) gp[c] += a.p2p_part[9 * (size_t)leaf + c];
        const int b = a.off[leaf], n = a.off[leaf + 1] - b;
        if (n == 0) continue;
        int ix, iy, iz;
        morton_decode((uint32_t)leaf, ix, iy, iz);
        const int iv[3] = {ix, iy, iz};
        double cen[3];
        for (int d = 0; d < 3; d++) {
            const float2 cc = sc->centre[d][iv[d]];
            cen[d] = (double)cc.x + (double)cc.y;
        }
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const float4 at = a.atoms[b + i], nf = a.near[b + i], ff = a.far[b + i];
            const double r[3] = {cen[0] + (double)at.x * h, cen[1] + (double)at.y * h, cen[2] + (double)at.z * h};
            const double qk = -(double)at.w * kf;
            const double F[3] = {qk * ((double)nf.y + (double)ff.y), qk * ((double)nf.z + (double)ff.z),
                                 qk * ((double)nf.w + (double)ff.w)};
            for (int x = 0; x < 3; x++)
                for (int y = 0; y < 3; y++) w[3 * x + y] += r[x] * F[y];
            for (int x = 0; x < 3; x++) {
                const float4 lf = a.lam_field[x][b + i];
                gf[3 * x + 0] += qk * (double)lf.y;
                gf[3 * x + 1] += qk * (double)lf.z;
                gf[3 * x + 2] += qk * (double)lf.w;
            }
        }
    }
    // block sums in a fixed order (per warp by shuffles, then warp 0 over the warps)
    __shared__ double red[8][27];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = 0; c < 27; c++) {
        double v = c < 9 ? w[c] : c < 18 ? gf[c - 9] : gp[c - 18];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 27) {
        double t = 0;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) t += red[ww][threadIdx.x];
        a.out[27 * (size_t)blockIdx.x + threadIdx.x] = t;
    }
}

void launch_virial_p2p(const P2PArgs& a, double* part, cudaStream_t s)
{
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    k_vir_p2p<<<a.nleaf, 128, 0, s>>>(a, part);
}

void launch_virial_m2l(const VirialM2LArgs& a, cudaStream_t s)
{
    long warps = 0;
    for (int k = 1; k <= a.depth; k++) warps += a.ncell[k];
    if (warps <= 0) return;
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    k_vir_m2l<<<(unsigned)((warps + 7) / 8), 256, sizeof(float) * 8 * a.Rpad, s>>>(a);
}

void launch_virial_root(const VirialRootArgs& a, cudaStream_t s)
{
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    k_vir_root<<<3, 256, sizeof(double) * a.R, s>>>(a);
}

void launch_virial_reduce(const VirialReduceArgs& a, int blocks, cudaStream_t s)
{
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
    k_vir_reduce<<<blocks, 256, 0, s>>>(a);
}

}  // namespace gbfmm
