// Shared definitions of the GB300 FMM library: Morton codes, real-representation
// indexing of expansions, error plumbing.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#ifndef GBFMM_HD
#define GBFMM_HD __host__ __device__ __forceinline__
#endif

namespace gbfmm {

constexpr double KE = 138.935457833;  // gmx::c_one4PiEps0 (units.h:110), kJ mol^-1 nm e^-2
constexpr int MAX_ORDER = 16;
constexpr int MAX_DEPTH = 7;

// Real representation of a complex expansion with conjugate symmetry: degree n
// occupies rows n*n .. n*n+2n: [Re(n,0), Re(n,1), Im(n,1), ..., Re(n,n), Im(n,n)].
GBFMM_HD int nreal(int P) { return (P + 1) * (P + 1); }
GBFMM_HD int ridx_re(int n, int m) { return n * n + (m == 0 ? 0 : 2 * m - 1); }
GBFMM_HD int ridx_im(int n, int m) { return n * n + 2 * m; }  // m >= 1
GBFMM_HD int rdeg(int r) {
    int n = 0;
    while ((n + 1) * (n + 1) <= r) n++;
    return n;
}

// Morton code of a cell at one level: per level one octant triple with the x bit
// highest, exactly the child numbering of CompleteBalancedOctree::build
// (tree.cpp:49-51, 85-92): octant = (x>c)<<2 | (y>c)<<1 | (z>c).
GBFMM_HD uint32_t spread3(uint32_t v) {
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x030000ff;
    v = (v | (v << 8)) & 0x0300f00f;
    v = (v | (v << 4)) & 0x030c30c3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
}
GBFMM_HD uint32_t compact3(uint32_t v) {
    v &= 0x09249249;
    v = (v | (v >> 2)) & 0x030c30c3;
    v = (v | (v >> 4)) & 0x0300f00f;
    v = (v | (v >> 8)) & 0x030000ff;
    v = (v | (v >> 16)) & 0x000003ff;
    return v;
}
GBFMM_HD uint32_t morton_encode(uint32_t ix, uint32_t iy, uint32_t iz) {
    return (spread3(ix) << 2) | (spread3(iy) << 1) | spread3(iz);
}
GBFMM_HD void morton_decode(uint32_t c, int& ix, int& iy, int& iz) {
    ix = (int)compact3(c >> 2);
    iy = (int)compact3(c >> 1);
    iz = (int)compact3(c);
}
// BFS index of the first cell of a level in the complete octree.
GBFMM_HD long level_base(int k) { return ((1L << (3 * k)) - 1) / 7; }

// Stored cells of one level along one axis: 2^(level - shift) (at least 1).
// A cubic box stores all 8^level cells of every level (shift 0 on every axis).
// A slab box with Lz = 2 Lx = 2 Ly is solved as the periodic virtual cube of edge
// Lz that holds it twice along x and twice along y (the same periodic charge
// density): the tree's root is that cube, and each level stores only the cells
// of the box itself (shift 1 along x and y), which are the Morton prefix
// [0, 8^level / 4) of every level >= 1; a cell outside it is the box cell at the
// same position modulo the box (periodic wrap per axis).
GBFMM_HD int grid_n(int level, int shift) { return level >= shift ? 1 << (level - shift) : 1; }
GBFMM_HD long grid_cells(int level, const int shift[3])
{
    return (long)grid_n(level, shift[0]) * grid_n(level, shift[1]) * grid_n(level, shift[2]);
}

#ifdef __CUDACC__
// Sums of FP32 products held as unevaluated FP32 pairs (hi + lo, about 48
// significant bits) with error-free transformations: the exact product by FMA
// (hi = a*b rounded, lo = fma(a, b, -hi)) and Knuth's two-sum.  On GB300 an FP64
// add waits ~64 cycles for its predecessor and the SM retires 2 FP64 lanes per
// clock, against 4 cycles and 128 lanes for FP32, so reductions run in this form
// and only their final value is converted to FP64.
struct f2sum {
    float hi, lo;
};
__device__ __forceinline__ f2sum f2s_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ f2sum f2s_add(f2sum a, f2sum b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
// Fixed butterfly over the warp: every lane ends with the same sum.
__device__ __forceinline__ f2sum f2s_warp_sum(f2sum v)
{
    for (int o = 16; o > 0; o >>= 1) {
        f2sum w;
        w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
        // the same operand order on both lanes of a pair: lower lane first
        v = (threadIdx.x & o) ? f2s_add(w, v) : f2s_add(v, w);
    }
    return v;
}
__device__ __forceinline__ double f2s_value(f2sum v) { return (double)v.hi + (double)v.lo; }
#endif

}  // namespace gbfmm
