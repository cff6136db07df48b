// Launch interface of the FMM device kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "common.cuh"

namespace gbfmm {

// One entry of a batched contraction: source cell relative to the target.
//   mode 0: same level, source = target coords + d
//   mode 1: parent level, source = parent coords + d
//   mode 2: child level, source = 2*target coords + d (d = child octant bits)
struct CEntry {
    int8_t dx, dy, dz, mode;
    int op;  // float offset of the packed operator
};

// One CTA job of a batched contraction.
struct CTask {
    int level;    // target level
    int octant;   // >= 0: targets are 8*(q0+t)+octant; < 0: targets are q0+t
    int q0;
    int ntgt;     // targets in this tile (<= tile size)
    int e_begin, e_end;
    int group;    // row group (work-item set) of this CTA
    int r0, r1;   // output rows written by this CTA
};

struct BlockInfo {
    int c0, off;
};

constexpr int CT_TILE = 64;   // targets per contraction CTA
constexpr int CT_WARPS = 8;
constexpr int CT_MAXI = 6;    // work items per warp (register accumulators)

struct ContractArgs {
    const float* ops;
    const CEntry* entries;
    const CTask* tasks;
    const int4* items;        // (blk, ca, cb, 0)
    const int* warp_begin;    // CT_WARPS+1
    const BlockInfo* blocks;  // per 8-row block
    float* src_lvl[8];
    float* dst_lvl[8];
    int R, Rpad, nblk;
    int periodic;
    int write_mode;           // 0 store, 1 add, 2 atomic add
    int shift[3];             // stored cells per axis of level l: grid_n(l, shift[d])
    const int* leaf_off;      // M2L: leaf offsets of the step (tiles of empty targets are skipped), or NULL
    int depth;                // leaf level
};

// Per-step constants that depend on the box, read by the kernels from device
// memory so that a captured graph can be replayed for a new box and new
// coordinate pointer without re-capture.
struct StepConst {
    const float* coords;                 // 3N coordinates of this step (device, or host memory the device reads in place)
    // where the finalize writes this step's results: the handle's device buffers,
    // or (a host call on a device that reaches pageable memory) its pinned host
    // buffers, written in place with no copy afterwards
    float* out_forces;                   // 3N, input order
    float* out_pots;                     // N
    double* out_energy;
    int* out_flags;                      // non-NULL: the finalize's last block copies the step's 4 flags here
    float inv_h;                         // 2^D / C (C: edge of the root cube)
    int copies;                          // copies of the box in the root cube (1 cubic, 4 slab)
    double coef;                         // 4 pi / (3 V), dipole correction (V: box volume)
    double box_len;                      // C, the edge of the root cube (nm): the period of a cubic box
    double inv_box_len;                  // 1 / C
    double box_centre[3];                // centre of the box (nm)
    int nd[3];                           // leaf cells per axis of the stored grid
    int pad_;
    float thresh[3][(1 << MAX_DEPTH) + 1];  // leaf boundaries rounded down to float (T[0] = -inf)
    float2 centre[3][1 << MAX_DEPTH];   // leaf centres as hi + lo floats
};

struct TreeArgs {
    const StepConst* sc;    // this step's constants (device memory, or the by-value launch's parameter)
    StepConst* sc_copy = nullptr;  // when set, block 0 copies *sc here for the step's later kernels
    const float* charges;   // N, input order
    int n;
    int depth;
    uint32_t* code;         // N leaf codes (input order)
    float4* uq;             // N scaled coords + charge (input order)
    int* counts;            // 8^D
    int* rank = nullptr;    // N: each body's arrival index in its leaf (the count's atomic), or none
    double* partials;       // per block: dipole (3) and total charge, FP32 pairs (hi, lo)
    int* flags;             // [0] non-finite input seen
    // Last-block epilogue (done NULL: none).  The last block to finish sums the
    // partials into sums[4] (fixed order) when sums != NULL and, when off != NULL,
    // writes the exclusive scan of counts into off[0..nleaf] and cursor[0..nleaf).
    // done is a counter that is zero when the kernel starts (and again at its end).
    int* done = nullptr;
    double* sums = nullptr;
    int* off = nullptr;
    int* cursor = nullptr;
    int nleaf = 0;
    // Read-only data of the later stages, prefetched into L2 by block 0 at the
    // start of the step (addresses 16-byte aligned, sizes rounded down to 16).
    static constexpr int MAX_PREFETCH = 8;
    const void* pf[MAX_PREFETCH] = {};
    unsigned long long pf_bytes[MAX_PREFETCH] = {};
    // Buffer of the step zeroed on the way (the local expansions, which the
    // far field accumulates into): zero_n4 float4s, or none when NULL.
    float4* zero = nullptr;
    long zero_n4 = 0;
};
// Leaf counts up to this size are scanned by the tree-key kernel's last block.
constexpr int TREE_EPILOGUE_MAX_LEAVES = 1 << 15;
// Caps of the grid-stride tree-key and finalize grids (their per-block partial
// sums are reduced by one warp): about four blocks per SM on a 152-SM GB300.
constexpr int TREE_MAX_BLOCKS = 608;
constexpr int FINAL_MAX_BLOCKS = 608;
int tree_blocks(int n);
int final_blocks(int n);

// Arguments of the per-system kernels that a batch also launches for many
// systems at once (one struct per system in device memory).
struct ScatterArgs {
    const uint32_t* code;
    int n;
    const int* off;
    const int* rank;
    int* tmp;
};
struct LeafSortArgs {
    const int* off;
    int nleaf;
    const int* tmp_idx;
    const float4* uq;
    int* order;
    float4* atoms;
    int* inv;
    int* counts;
    int* edge;
};
struct P2MArgs {          // P2M of the leaves (and, fused, the M2M of their parents)
    const int* off;
    int nleaf;
    const float4* atoms;
    float* M;
    float* Mp;            // parents (fused form)
    const float* At;      // transposed M2M operators (fused form)
    int Rpad;
};
struct L2PArgs {
    const int* off;
    int nleaf;
    const float4* atoms;
    const float* L;
    int Rpad;
    float4* field;
};
struct M2MArgs {
    const float* Mc;
    float* Mp;
    const float* At;
    int nparent, R, Rpad;
};

extern std::atomic<long> g_kernel_launches;

// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount,
// cached per device).
int sm_count();

// by_value: the step's constants travel as a parameter of the launch (a.sc is
// ignored; a.sc_copy receives them); else the kernel reads them at a.sc.
void launch_tree_keys(const TreeArgs& a, cudaStream_t s, const StepConst* by_value = nullptr);
const void* tree_keys_sc_kernel();  // the by-value kernel (to find its node in a captured graph)
void launch_exclusive_scan(const int* in, int* out, int n, int* scratch, cudaStream_t s);
void launch_scatter(const uint32_t* code, int n, int* cursor, int* tmp_idx, cudaStream_t s);
// The same without atomics: tmp_idx[off[code[i]] + rank[i]] = i (TreeArgs::rank).
// The launchers below that take 'pdl' launch, when it is set, as programmatic
// dependents of the previous kernel of s (launch_k): the kernel may start while
// that one finishes and waits for it (pdl_wait) before it touches its data.
void launch_scatter_ranked(const uint32_t* code, int n, const int* off, const int* rank, int* tmp_idx,
                           cudaStream_t s, bool pdl = false);
// Also zeroes counts[0..nleaf) (consumed by then) when counts != NULL.
// inv[input index] = sorted position (the inverse of order); edge[leaf] (when
// not NULL) = 1 if a body of the leaf lies on or near its faces or outside it.
void launch_leaf_sort(const int* offsets, int nleaf, int* tmp_idx, const float4* uq, const uint32_t* code, int* order,
                      float4* atoms, int* inv, int* counts, cudaStream_t s, int* edge = nullptr, bool pdl = false);
void launch_p2m(int P, const int* offsets, int nleaf, const float4* atoms, float* M_leaf, int Rpad, cudaStream_t s,
                bool pdl = false);
// P2M of the leaves and M2M of their parents in one launch (8 sibling leaves per
// CTA).  Returns false, launching nothing, when the order's shared memory does
// not fit or nleaf is not a multiple of 8.
bool launch_p2m_m2m(int P, const int* offsets, int nleaf, const float4* atoms, float* M_leaf, float* M_parent,
                    const float* At, int Rpad, cudaStream_t s, bool pdl = false);
void launch_l2p(int P, const int* offsets, int nleaf, const float4* atoms, const float* L_leaf, int Rpad, float4* field,
                cudaStream_t s);
// Near field.  variant = shape + 3 * persistence: shape = the warp-step shape
// (0: 8 targets x 4 source lanes, 1: 4 x 8, 2: 16 x 2); persistence 0 = one CTA
// per leaf, 1..4 = (persistence + 1) CTAs per SM walking the leaves through
// *counter (zero at launch).  Chosen by the autotuner; all give the same sums up
// to the order of the additions.  Variants 15 and 16: one CTA per leaf, up to 4
// targets per thread, shapes 8 x 4 and 4 x 8.
struct P2PArgs {
    const int* off;           // leaf offsets (nleaf + 1)
    int nleaf, periodic;
    int nd[3];                // leaf cells per axis (periodic wrap of the stencil)
    const float4* atoms;      // sorted (u, q)
    const int* stencil;       // nst offsets (3 ints), the zero offset first
    int nst;
    float4* field;            // sorted near field (phi, grad), scaled units
    const int* leaf_edge;     // per leaf: a body on or near its faces or outside it (from the leaf sort)
    int* err = nullptr;              // bit 2: a bounded wait on the staging copies gave up
    uint32_t wait_limit = 1u << 24;  // polls of that wait
};
int p2p_variants();
// Near fields of many systems in one persistent launch (per_sm CTAs per SM).
struct P2PBatchArgs {
    const P2PArgs* sys;  // nsys (device)
    const int* first;    // nsys + 1 prefix sums of the systems' leaf counts (device)
    int nsys, nitems;
    int* counter;        // zero at launch
};
// shape: 0 8 targets x 4 source lanes, 1 4 x 8, 2 16 x 2, 3 and 4 the shapes 8 x 4
// and 4 x 8 with up to 4 targets per thread; per_sm 1..5 resident CTAs per SM
// walking the queue, or 0: one CTA per queue item.
int p2p_batch_shapes();
void launch_p2p_batch(const P2PBatchArgs& b, int shape, int per_sm, cudaStream_t s);
void launch_p2p(const P2PArgs& a, int variant, cudaStream_t s, int* counter);
void launch_contract(const ContractArgs& a, int ntasks, cudaStream_t s);
// Fused downward pass (depth >= 2): L2L of levels 2..depth and L2P, one launch.
struct DownArgs {
    int nparent;              // stored cells of level depth-1 (one CTA each)
    const int* off;
    const float4* atoms;
    const float* L[8];        // per level: L~ rows holding their M2L part (level 1: complete)
    const float* l2l_t;       // 8 transposed R x R scaled L2L operators
    float4* field;            // sorted far field (phi, grad), scaled units
    int depth, Rpad;
    int* err = nullptr;              // bit 1: the bounded wait on the staged operators gave up
    uint32_t wait_limit = 1u << 24;  // polls of that wait
};
void launch_down(int P, const DownArgs& a, cudaStream_t s, bool pdl = false);
// Dynamic shared memory of the downward pass of order P: the 8 L2L operators,
// staged by one bulk copy where they fit (orders up to 6), else 0 (read from L2).
size_t down_smem_bytes(int P);

// One level of M2M (nparent parents from their 8 children each); At = 8
// transposed R x R scaled operators.
void launch_m2m(const float* M_child, float* M_parent, const float* At, int nparent, int R, int Rpad, cudaStream_t s,
                bool pdl = false);

struct RootArgs {
    int R, Rpad;
    const double* m2m;      // 8 blocks of R x R, block o at o * ((R^2 + 1) & ~1)
    const double* l2l;      // 8 x R x R
    const double* lattice;  // R x R (allocated to an even count)
    const float* M1;        // level-1 multipoles (8 rows)
    double* M0;             // root multipole (FP64)
    double* L0;             // root local (FP64)
    float* M0f;             // FP32 copy of the root multipole (level-0 row)
    float* L1;              // level-1 locals (8 rows)
    const StepConst* sc;
    int images;
    int n1 = 8;             // stored level-1 cells: octants 0..n1-1 (8 cubic, 2 slab)
};
void launch_root_lattice(const RootArgs& a, cudaStream_t s);
void launch_root_l2l(const RootArgs& a, cudaStream_t s);

// The upper tree in one launch of 8 CTAs (one per level-1 cell).  For
// R <= TOP_STAGE_MAX_R (orders up to 6) the operators are staged in shared memory
// and the launch does the M2M from level 'from' (3, 2, or 1 = level 1 already
// complete) up to level 1; for larger R only from = 1 is allowed (the M2M levels
// take launch_m2m).  Then the FP64 root M2M and, when 'lattice' is set, the
// lattice operator (else launch_top follows with launch_root_lattice).  Same
// arithmetic as launch_m2m per level, the root M2M and launch_root_lattice.
struct TopArgs {
    RootArgs root;
    int from;
    int lattice;          // 1: the last CTA applies the lattice operator (R <= TOP_LATTICE_MAX_R)
    const float* Min;     // multipoles of level 'from' (from >= 2)
    float* M2;            // level-2 multipoles (written when from = 3)
    float* M1;            // level-1 multipoles (written when from >= 2, read when from = 1)
    const float* m2m_t;   // FP32 M2M operator, [octant][column][row]
    double* part;         // 8 x R x 4 FP64 partial sums of the root M2M
    const double* tree_part;  // the tree-key kernel's per-block dipole/charge partials (FP32 pairs)
    int tree_nblocks;
    double* sums;         // out: dipole (3) and total charge, FP64
    float* fconst;        // out: FP32 dipole-correction constants of the finalize (4)
    double inv_natoms;    // 1 / max(atoms, 1)
    int* done;            // zero at launch
    int* err;             // bit 1: the bounded wait for the staged copies gave up
    // CTA g < root.n1 owns stored level-1 cell g and the root-M2M shares of the
    // octants o with (o & umask) == g (umask 7 cubic; 1 slab: the x and y halves
    // of the root cube repeat the box)
    int umask = 7;
    uint32_t wait_limit = 1u << 24;  // polls of the bounded wait
};
constexpr int TOP_STAGE_MAX_R = 49;
constexpr int TOP_LATTICE_MAX_R = TOP_STAGE_MAX_R;  // larger: the multi-CTA k_root_lattice
size_t top_smem_bytes(int R);
void launch_top(const TopArgs& a, cudaStream_t s, bool pdl = false);

// Bounded-wait probe: one warp waits on an mbarrier that nothing completes,
// with no copies or MMAs in flight; after 'polls' polls the wait gives up and
// sets bit 1 of *err.  Exercises the give-up path of the bounded waits.
void launch_wait_probe(uint32_t polls, int* err, cudaStream_t s);

// ---- batched launches: one launch of a kernel for many systems (CTA b runs block
// b - first[s] of system s; args = one struct per system in device memory).
enum class BatchKernel {
    TREE_KEYS, SCATTER, LEAF_SORT, P2M, P2M_M2M, L2P, DOWN, M2M, TOP_STAGED, TOP_UNSTAGED, ROOT_LATTICE, FINALIZE,
    TC_GRIDS, M2L_TC
};
// P: the order (templated kernels); smem: dynamic shared memory of the launch.
void launch_batch(BatchKernel k, int P, const void* args, const int* first, int nsys, int nblocks, size_t smem,
                  cudaStream_t s);
// The tensor-core kernels (m2l_tc.cu).
void launch_batch_tc(BatchKernel k, const void* args, const int* first, int nsys, int nblocks, size_t smem,
                     cudaStream_t s);
size_t p2m_smem_bytes(int P);        // dynamic shared memory of k_p2m<P>
size_t p2m_m2m_smem_bytes(int P);    // of k_p2m_m2m<P> (0: the fused kernel is not used for P)
int p2m_warps(int P);                // warps (leaves) per CTA of k_p2m<P>

// ---- virial (virial.cu): the image-shift terms of Xi = -1/2 sum_pairs r (x) F
constexpr int VIR_MAXR = 320;  // rows of the largest expansion (order 16: 289)
struct VirialM2LArgs {
    int depth, R, Rpad;
    long ncell[MAX_DEPTH + 1];     // stored cells per level
    int shift[3];                  // stored cells per axis: grid_n(level, shift[d])
    const CEntry* entries;         // M2L stencil entries, op = class index
    int e_first[2][8], e_count[2][8];  // [level 1 | levels >= 2][target octant]
    const float* ops;              // per class R x R FP32, [column][row]
    const float* M[MAX_DEPTH + 1]; // multipoles per level (level 0: the root's FP32 copy)
    float* lam[3][MAX_DEPTH + 1];  // shift-weighted locals per axis and level
};
struct VirialRootArgs {
    int R, Rpad, n1;
    const double* lat_shift;       // 3 x R x R (lattice_shift_operators)
    const double* M0;              // root multipole (FP64)
    const double* l2l;             // 8 x R x R root L2L (FP64)
    double scale[3];               // root-cube edge / period along the axis
    float* lam1[3];                // level-1 rows of the three shift-weighted locals
};
struct VirialReduceArgs {
    const StepConst* sc;
    int nleaf;
    const int* off;
    const float4* atoms;           // sorted (u, q)
    const float4 *near, *far;      // sorted fields of the step
    const float4* lam_field[3];    // sorted fields of the shift-weighted locals
    const double* p2p_part;        // 9 per leaf (k_vir_p2p)
    double* out;                   // 27 per block: sum r (x) F, sum F[Lambda], sum of the p2p partials
};
void launch_virial_p2p(const P2PArgs& a, double* part, cudaStream_t s);
void launch_virial_m2l(const VirialM2LArgs& a, cudaStream_t s);
void launch_virial_root(const VirialRootArgs& a, cudaStream_t s);
void launch_virial_reduce(const VirialReduceArgs& a, int blocks, cudaStream_t s);

struct FinalArgs {
    const StepConst* sc;
    int n;
    const float4* atoms;     // sorted (u, q)
    const int* inv;          // input index -> sorted position
    const float4* near;      // sorted (phi, grad) near field, scaled units
    const float4* far;       // sorted far field, scaled units
    const float* fconst;     // q*ke*coef*M (3) and ke*coef*|M|^2/N, FP32 (written by k_top)
    const int* flags;        // the step's 4 flags (device), copied to sc->out_flags when that is set
    double* partials;        // per block: 0.5 * sum q * pot as an FP32 pair (hi, lo)
    int* done = nullptr;     // zero at start: the last block sums the partials into *sc->out_energy and re-zeroes it
    int* zero_after = nullptr;  // a counter of the step (the P2P queue) that the last block also re-zeroes
};
void launch_finalize(const FinalArgs& a, cudaStream_t s);

}  // namespace gbfmm
