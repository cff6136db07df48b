// Tensor-core (tcgen05) M2L: launch interface, the host-side chunk plan and the
// layout of the bf16 source grids that the TMA engine reads.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "kernels.h"

namespace gbfmm {

// Orders of the tensor-core M2L: up to 12 (a multipole row of 169 coefficients,
// three 64-element K atoms; one pipeline stage of the split-precision form fits
// a CTA's shared memory at orders 11-12, two or more of the single product).
constexpr int TC_MAX_ORDER = 12;
constexpr int TC_MAXCHUNK = 8;
constexpr int TC_TILE = 128;     // MMA M: rows of the target tile
constexpr int TC_MAXSTAGE = 8;   // pipeline stages (operands of one entry each)
constexpr int TC_THREADS = 128;  // producer lane, MMA lane, 4 epilogue warps
constexpr int TC_HALO = 2;       // halo of the source grids (cells of the grid)
constexpr int TC_MAXLEV = 8;
constexpr int TC_MAXENT = 256;
#ifndef TC_GROUP_DEFAULT
#define TC_GROUP_DEFAULT 1
#endif
constexpr int TC_NSPLIT = 4;     // entry splits 1, 2, 4, 8 of a tile's stencil (autotuned)   // stencil entries of one task (the stencils have at most 182)

// Degree chunks of the M2L operator: chunk c covers output rows [row0, row0+rows)
// (whole degrees j0..j1), MMA N = n (rows padded to 16), K = k (inputs of degree
// <= P-j0, padded to 16), accumulator columns [col, col+n) of TMEM, operator image
// at byte offset img inside one class image.
struct TcPlan {
    int P = 0, nchunk = 0;
    int n[TC_MAXCHUNK], k[TC_MAXCHUNK], col[TC_MAXCHUNK], row0[TC_MAXCHUNK], rows[TC_MAXCHUNK], img[TC_MAXCHUNK];
    int img_bytes = 0;   // bytes of one (hi or lo) class image
    int k_atoms = 0;     // 64-element (128-byte) K atoms of the A tile
    int tmem_cols = 0;   // power of two >= sum of n
};

TcPlan make_tc_plan(int P);
// Appends the hi and lo images of one R x R operator (row-major FP64) to 'out'.
void append_tc_image(const TcPlan& pl, int R, const double* A, std::vector<uint8_t>& out);

// Source grids.  Every grid row holds KP = 64 * k_atoms bf16 coefficients of one
// cell (zero past R), hi and lo splits in two arrays of the same layout.  With
// n_d stored cells of the level along axis d (grid_n):
//   parity grid of level k >= 1 (same-level sources): [par][zh][yh][xh][KP] with
//     W_d = ceil(n_d / 2) + 2 TC_HALO, cell x = 2 (xh - TC_HALO) + px,
//     par = px + 2 py + 4 pz;
//   natural grid of level k >= 0 (parent-level sources): [z][y][x][KP] with
//     W_d = n_d + 2 TC_HALO, cell x = x' - TC_HALO.
// Halo cells hold the periodic images (or zeros without periodicity), so the
// sources of a tile of same-octant targets for one stencil entry form one
// rectangular box: a single TMA tile load.
struct TcGrids {
    int KP = 0;
    long rows = 0;
    long p_row0[TC_MAXLEV] = {}, n_row0[TC_MAXLEV] = {};
    int p_w[TC_MAXLEV][3] = {}, n_w[TC_MAXLEV][3] = {};
};
TcGrids tc_grid_layout(int D, int k_atoms, const int shift[3]);

// Target tile of level k: a box of bx x by x bz parent cells (one octant).
void tc_tile_shape(int level, const int shift[3], int& bx, int& by, int& bz);
int tc_tiles(int level, const int shift[3]);
// Target octants of level k that the stored grid holds (all 8 except at levels
// where an axis has one cell: that axis's octant bit is then 0).
bool tc_octant_stored(int level, const int shift[3], int octant);

struct TcGridArgs {
    int ngrid = 0;
    long row0[2 * TC_MAXLEV];
    int level[2 * TC_MAXLEV], parity[2 * TC_MAXLEV], W[2 * TC_MAXLEV][3], n[2 * TC_MAXLEV][3];
    const float* src[2 * TC_MAXLEV];  // FP32 rows of that level (Morton order)
    int R, Rpad, KP, periodic;
    long rows;                        // rows [row_begin, rows) of the grid buffers are converted
    long row_begin = 0;
    __nv_bfloat16 *hi, *lo;           // lo may be NULL (one product)
    // Root L2L, run by extra blocks of the same launch (before the M2L adds to
    // level 1): L1[o][r] += sum_c l2l[o][r][c] L0[c] in FP64, one warp per (o, r),
    // the arithmetic of k_root_l2l.  Skipped when root_l2l is NULL.
    const double* root_l2l = nullptr;
    const double* L0 = nullptr;
    float* L1 = nullptr;
    int root_R = 0;
    int root_n1 = 8;  // stored level-1 cells
};
void launch_tc_grids(const TcGridArgs& g, cudaStream_t s, bool pdl = false);  // pdl: as launch_down
long tc_grids_blocks(const TcGridArgs& g);  // CTAs of one system's launch_tc_grids

struct alignas(64) TcArgs {
    CUtensorMap p_hi[TC_MAXLEV], p_lo[TC_MAXLEV];  // parity grids (level k)
    CUtensorMap n_hi[TC_MAXLEV], n_lo[TC_MAXLEV];  // natural grids (level k)
    const uint8_t* bimg;         // class images: [class][hi | lo]
    const CEntry* entries;       // op = class index
    const CTask* tasks;          // level, octant, q0 = tile index, entry range
    float* dst_lvl[TC_MAXLEV];
    int* err;                    // bit 1: a bounded wait gave up
    uint32_t wait_limit;         // polls of each bounded wait (WAIT_POLLS_DEFAULT)
    int Rpad;
    int k_atoms, img_bytes, tmem_cols, nchunk;
    int nprod;                   // 3: hi*hi + hi*lo + lo*hi, 1: hi*hi
    int nstage;                  // pipeline stages, 2..TC_MAXSTAGE (tc_pick_stages)
    int group;                   // stencil entries per stage (one expect_tx, one wait, one commit)
    int atomic;                  // 1: atomicAdd into L (split entry ranges), 0: plain add
    int shift[3];                // stored cells per axis of level l: grid_n(l, shift[d])
    const int* leaf_off;         // leaf offsets of the step (tiles of empty targets are skipped), or NULL
    int depth;                   // leaf level
    int chunk_n[TC_MAXCHUNK], chunk_k[TC_MAXCHUNK], chunk_col[TC_MAXCHUNK], chunk_row0[TC_MAXCHUNK],
        chunk_rows[TC_MAXCHUNK], chunk_img[TC_MAXCHUNK];
};

// Encodes the tensor maps of the grids (hi, and lo when lo != NULL) into a.
// Returns false when the driver's encoder is unavailable or refuses a map.
bool tc_encode_maps(TcArgs& a, int D, const TcGrids& g, void* hi, void* lo);
size_t tc_smem_bytes(const TcArgs& a);
size_t tc_stage_bytes(int k_atoms, int img_bytes, int nprod);  // the operands of one entry
int tc_pick_stages(int k_atoms, int img_bytes, int nprod);
int tc_max_stages(int k_atoms, int img_bytes, int nprod);  // most that fit one CTA's shared memory
void launch_m2l_tc(const TcArgs& a, int ntasks, cudaStream_t s, bool pdl = false);  // pdl: as launch_down

}  // namespace gbfmm
