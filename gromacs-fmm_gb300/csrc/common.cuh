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

}  // namespace gbfmm
