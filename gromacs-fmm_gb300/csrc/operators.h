// Host-side (FP64) construction of the FMM translation operators, interaction
// stencils and reference-ordered interaction lists.
#pragma once

#include <cstdint>
#include <vector>

namespace gbfmm {

// ---- harmonics (FP64, Cartesian recurrences; packed index n*(n+1)/2+m, m>=0)
void harm_regular(int P, const double d[3], double* re, double* im);
void harm_singular(int P, const double d[3], double* re, double* im);

// ---- dense real operators (R x R row-major, R = (P+1)^2) in unscaled units
void m2m_matrix(int P, const double dx[3], double* A);   // dx = parent centre - child centre
void l2l_matrix(int P, const double dX[3], double* A);   // dX = child centre - parent centre
void m2l_matrix(int P, const double dX[3], double* A);   // dX = target centre - source centre

// M2L classes: kind 0 = same level, Delta = v (target cell units);
//              kind 1 = source one level coarser, Delta = v/2 (target cell units).
struct M2LClass {
    int kind;
    int v[3];
};

// One entry of a per-(level type, target octant) M2L stencil.
//   mode 0: source at the target's level, source coords = target coords + d
//   mode 1: source at the parent level,   source coords = parent coords + d
struct StencilEntry {
    int mode;
    int d[3];
    int cls;  // index into the class table
};

struct Stencils {
    // [0] = level 1 (parent is the root: 27 periodic shifts), [1] = levels >= 2
    std::vector<StencilEntry> m2l[2][8];
    std::vector<M2LClass> classes;
    std::vector<int> p2p;  // 81 offsets d (3 ints each): source leaf = target leaf + d
};

// Builds the stencils of the reference traversal (traverser.cpp:88-214) for a
// complete periodic octree with MAC scale theta.
Stencils build_stencils(double theta);

// Scaled operators (cell size of the target level = 1):
//   M~_n = M_n / h^n,   L~_j = L_j * h^(j+1)
void scaled_m2m(int P, int octant, double* A);
void scaled_l2l(int P, int octant, double* A);
void scaled_m2l(int P, const M2LClass& c, double* A);
// Periodic lattice operator L~_root = A M~_root (root cell size 1), FP64.
void lattice_operator(int P, int images, double* A);
// The same lattice weighted by each far image box's index n_a (periods), a = x, y, z:
// 3 consecutive R x R matrices (the virial's image-shift term).
void lattice_shift_operators(int P, int images, double* A3);

// Packed layout of an operator for the SIMT contraction kernel: rows in blocks of
// 8; block b covers input columns [c0[b], c1[b]); stored as (c1-c0) x 8 floats.
enum OpType { OP_M2L = 0, OP_M2M = 1, OP_L2L = 2 };
struct PackPlan {
    int P = 0, R = 0, nblk = 0, packed = 0;
    std::vector<int> c0, c1, off;
};
PackPlan make_pack_plan(int P, OpType t);
void pack_operator(const PackPlan& plan, const double* A, float* out);

// Work items of one contraction: (block, column range), partitioned across warps.
struct WorkItem {
    int16_t blk, ca, cb, pad;
};
struct WorkPartition {
    int groups = 0;
    std::vector<WorkItem> items;
    std::vector<int> warp_begin;  // groups x (n_warps + 1)
    std::vector<int> row0, row1;  // output rows of each group
};
bool make_work_items(const PackPlan& plan, int n_warps, int groups, int max_items, WorkPartition& out);

// Reference-ordered interaction lists for a complete tree of depth D.
struct RefLists {
    std::vector<int> tgt, src, off;  // off: 3 ints per entry, in units of the period
};
void emit_lists(const Stencils& st, int D, int images, RefLists& p2p, RefLists& m2l);

}  // namespace gbfmm
