// Tree build that allocates nothing: gbfmm_tree_build_noalloc.
//
// Some callers cannot allocate device memory when they call in: an MD engine
// whose own pool reserved the GPU's memory at start-up (a cudaMalloc inside the
// library would then fail mid-run), or a time-stepping loop that must not call
// cudaMalloc because it can synchronise the whole device.  For them this entry
// point runs the
// same tree kernels as gbfmm_execute (keys, counting sort, stable leaf order)
// with every scratch buffer carved out of one file-scope static device array of
// fixed size.  The caller passes the inputs (coordinates, charges) and the
// outputs (body order, leaf offsets) as device pointers.
//
// Limits: at most GBFMM_NOALLOC_MAX_ATOMS bodies and depth GBFMM_NOALLOC_MAX_DEPTH.
// Every GPU that loads the library holds the array (about 3 MB) until the
// process exits.  All calls share the array and it keeps the last call's
// contents; the counters that must start at zero are cleared on every call.
// Calls that overlap on the GPU (different streams, or different host threads)
// race on the shared scratch: order them.
//
// The array's device address is looked up (cudaGetSymbolAddress, with the
// device current) on the first call in each CUDA context and kept for that
// context; a call from a new context (after cudaDeviceReset, say) looks it up
// again.  The box-dependent constants reach the device as a kernel argument
// (copied at launch), not by a copy from host memory.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/gbfmm.h"
#include "common.cuh"
#include "kernels.h"

using namespace gbfmm;

namespace {

constexpr int NA = GBFMM_NOALLOC_MAX_ATOMS;
constexpr int NL = 1 << (3 * GBFMM_NOALLOC_MAX_DEPTH);

// byte offsets of the scratch pieces inside the static array (256-byte aligned)
constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t OFF_SC = 0;
constexpr size_t OFF_CODE = al(OFF_SC + sizeof(StepConst));
constexpr size_t OFF_UQ = al(OFF_CODE + sizeof(uint32_t) * NA);
constexpr size_t OFF_TMP = al(OFF_UQ + sizeof(float4) * NA);
constexpr size_t OFF_ATOMS = al(OFF_TMP + sizeof(int) * NA);
constexpr size_t OFF_LEAF = al(OFF_ATOMS + sizeof(float4) * NA);
constexpr size_t OFF_COUNTS = al(OFF_LEAF + sizeof(int) * NA);
constexpr size_t OFF_CURSOR = al(OFF_COUNTS + sizeof(int) * (NL + 1));
constexpr size_t OFF_BSUM = al(OFF_CURSOR + sizeof(int) * (NL + 1));
constexpr size_t OFF_PART = al(OFF_BSUM + sizeof(int) * (NL / 2048 + 2));
constexpr size_t OFF_FLAGS = al(OFF_PART + sizeof(double) * 4 * TREE_MAX_BLOCKS);
constexpr size_t SCRATCH_BYTES = al(OFF_FLAGS + sizeof(int) * 4);

static __device__ __align__(256) unsigned char g_tree_scratch[SCRATCH_BYTES];

// Status only: this entry point reports through its return value.
int err(int code, const char*) { return code; }

// Device address of g_tree_scratch per device, looked up with that device
// current (the host-side symbol is only a stand-in) and kept together with the
// context it belongs to: a new context on the device gets a new lookup.
std::mutex g_mu;
unsigned char* g_addr[64] = {};
CUcontext g_ctx[64] = {};

typedef CUresult (*ctx_get_current_fn)(CUcontext*);

// cuCtxGetCurrent through the runtime's driver entry point (no link to libcuda).
CUcontext current_context()
{
    static ctx_get_current_fn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<ctx_get_current_fn>(p);
        else
            cudaGetLastError();
    }
    CUcontext c = nullptr;
    if (fn) fn(&c);
    return c;
}

// Writes the step constants into the scratch: the constants travel as a kernel
// argument (copied when the kernel is launched).
__global__ void k_store_step_const(const StepConst sc, StepConst* dst)
{
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&sc);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    for (int i = threadIdx.x; i < (int)(sizeof(StepConst) / 4); i += blockDim.x) d[i] = s[i];
}
static_assert(sizeof(StepConst) % 4 == 0, "StepConst is copied in 4-byte words");

}  // namespace

extern "C" int gbfmm_tree_build_noalloc(const void* d_coords, const void* d_charges, int natoms, const float* box,
                                        int max_depth, void* d_order, void* d_leaf_offsets, void* stream)
{
    if (natoms < 0 || natoms > NA) return err(GBFMM_ERR_ARG, "natoms outside [0, GBFMM_NOALLOC_MAX_ATOMS]");
    if (max_depth < 1 || max_depth > GBFMM_NOALLOC_MAX_DEPTH)
        return err(GBFMM_ERR_ARG, "max_depth outside [1, GBFMM_NOALLOC_MAX_DEPTH]");
    if (!box || !d_leaf_offsets || (natoms > 0 && (!d_coords || !d_charges || !d_order)))
        return err(GBFMM_ERR_ARG, "NULL argument");
    for (int i = 0; i < 9; i++)
        if (!std::isfinite(box[i])) return err(GBFMM_ERR_BOX, "box entry is not finite");
    if (!(box[0] > 0) || box[1] != 0 || box[2] != 0 || box[3] != 0 || box[5] != 0 || box[6] != 0 || box[7] != 0 ||
        box[4] != box[0] || box[8] != box[0])
        return err(GBFMM_ERR_BOX, "box must be cubic with a positive edge");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return err(GBFMM_ERR_CUDA, "no CUDA device is current");
    }
    unsigned char* base;
    {
        const CUcontext ctx = current_context();
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev] || !ctx || g_ctx[dev] != ctx) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_tree_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return err(GBFMM_ERR_CUDA, "cudaGetSymbolAddress of the tree scratch failed");
            }
            g_addr[dev] = (unsigned char*)p;
            g_ctx[dev] = current_context();  // the lookup made the runtime's context current
        }
        base = g_addr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int D = max_depth, nd = 1 << D, nleaf = 1 << (3 * D);
    // box-dependent constants, as gbfmm_execute computes them
    StepConst sc;
    std::memset(&sc, 0, sizeof(sc));
    const double L = (double)box[0];
    sc.coords = (const float*)d_coords;
    sc.inv_h = (float)(nd / L);
    sc.coef = 4.0 * M_PI / (3.0 * L * L * L);
    sc.box_len = L;
    sc.inv_box_len = 1.0 / L;
    sc.copies = 1;
    for (int d = 0; d < 3; d++) {
        sc.nd[d] = nd;
        sc.box_centre[d] = L / 2;
    }
    for (int d = 0; d < 3; d++) {
        const double lo = (double)box[4 * d] / 2 - L / 2;
        sc.thresh[d][0] = -INFINITY;
        for (int j = 1; j < nd; j++) {
            double b = lo + L * j / nd;
            float f = (float)b;
            if ((double)f > b) f = std::nextafter(f, -INFINITY);
            sc.thresh[d][j] = f;
        }
        sc.thresh[d][nd] = INFINITY;
        for (int j = 0; j < nd; j++) {
            double c = lo + L * (2 * j + 1) / (2.0 * nd);
            float hi = (float)c;
            sc.centre[d][j] = make_float2(hi, (float)(c - (double)hi));
        }
    }
    StepConst* d_sc = (StepConst*)(base + OFF_SC);
    int* counts = (int*)(base + OFF_COUNTS);
    int* cursor = (int*)(base + OFF_CURSOR);
    int* off = (int*)d_leaf_offsets;
    k_store_step_const<<<1, 256, 0, s>>>(sc, d_sc);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(int) * (nleaf + 1), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + OFF_FLAGS, 0, sizeof(int) * 4, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return err(GBFMM_ERR_CUDA, cudaGetErrorString(e));
    }
    if (natoms > 0) {
        TreeArgs ta;
        ta.sc = d_sc;
        ta.charges = (const float*)d_charges;
        ta.n = natoms;
        ta.depth = D;
        ta.code = (uint32_t*)(base + OFF_CODE);
        ta.uq = (float4*)(base + OFF_UQ);
        ta.counts = counts;
        ta.partials = (double*)(base + OFF_PART);
        ta.flags = (int*)(base + OFF_FLAGS);
        launch_tree_keys(ta, s);
    }
    launch_exclusive_scan(counts, off, nleaf, (int*)(base + OFF_BSUM), s);
    e = cudaMemcpyAsync(cursor, off, sizeof(int) * nleaf, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return err(GBFMM_ERR_CUDA, cudaGetErrorString(e));
    }
    launch_scatter((const uint32_t*)(base + OFF_CODE), natoms, cursor, (int*)(base + OFF_TMP), s);
    launch_leaf_sort(off, nleaf, (int*)(base + OFF_TMP), (const float4*)(base + OFF_UQ),
                     (const uint32_t*)(base + OFF_CODE), (int*)d_order, (float4*)(base + OFF_ATOMS),
                     (int*)(base + OFF_LEAF), nullptr, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return err(GBFMM_ERR_CUDA, cudaGetErrorString(e));
    return GBFMM_OK;
}
