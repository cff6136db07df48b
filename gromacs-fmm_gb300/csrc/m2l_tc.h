// Tensor-core (tcgen05) M2L: launch interface and the host-side chunk plan.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "kernels.h"

namespace gbfmm {

constexpr int TC_KMAX = 128;     // length of a split (bf16) multipole row; orders P <= 10
constexpr int TC_MAX_ORDER = 10;
constexpr int TC_MAXCHUNK = 8;
constexpr int TC_TILE = 128;     // targets per CTA (MMA M)
constexpr int TC_MAXSTAGE = 4;   // pipeline stages (operands of one entry each)
constexpr int TC_THREADS = 160;  // 4 producer warps + 1 MMA warp

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

struct TcArgs {
    const __nv_bfloat16* mh[8];  // per level: split multipole rows (hi), TC_KMAX bf16 each
    const __nv_bfloat16* ml[8];  // (lo)
    const uint8_t* bimg;         // class images: [class][hi | lo]
    const CEntry* entries;       // op = class index
    const CTask* tasks;
    float* dst_lvl[8];
    int* err;                    // bit 1: a bounded wait gave up
    int Rpad;
    int k_atoms, img_bytes, tmem_cols, nchunk;
    int nprod;                   // 3: hi*hi + hi*lo + lo*hi, 1: hi*hi
    int nstage;                  // pipeline stages, 2..TC_MAXSTAGE (tc_pick_stages)
    int periodic;
    int atomic;                  // 1: atomicAdd into L (split entry ranges), 0: plain add
    int chunk_n[TC_MAXCHUNK], chunk_k[TC_MAXCHUNK], chunk_col[TC_MAXCHUNK], chunk_row0[TC_MAXCHUNK],
        chunk_rows[TC_MAXCHUNK], chunk_img[TC_MAXCHUNK];
};

size_t tc_smem_bytes(const TcArgs& a);
size_t tc_stage_bytes(int k_atoms, int img_bytes, int nprod);
int tc_pick_stages(int k_atoms, int img_bytes, int nprod);
void launch_m2l_tc(const TcArgs& a, int ntasks, cudaStream_t s);
void launch_split_bf16(const float* M, int Rpad, int R, long nrows, void* hi, void* lo, cudaStream_t s);

}  // namespace gbfmm
