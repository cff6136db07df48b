// Host orchestration and C ABI of the GB300 FMM (include/gbfmm.h).
//
// One handle = one system.  Everything that depends only on (order, depth,
// images) -- operators, stencils, contraction task lists -- is built and uploaded
// once at create time; device buffers are sized once (no per-step allocation,
// unlike GPUSolver::solve, src/gromacs/zeta_fmm/gpu_solver.cu:79-98, 258-270).
// Per step only the box-dependent constants (a few KB) change: they travel as a
// parameter of the step's first kernel, and the whole step is replayed from a
// captured CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <new>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbfmm.h"
#include "async.cuh"
#include "common.cuh"
#include "kernels.h"
#include "m2l_tc.h"
#include "operators.h"

using namespace gbfmm;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(e_ == cudaErrorMemoryAllocation ? GBFMM_ERR_NOMEM : GBFMM_ERR_CUDA, "%s: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);                             \
    } while (0)

// Operator tables shared by all handles of the same (order, images).
struct OpTables {
    int P = 0, images = -1, R = 0, Rpad = 0;
    Stencils st;
    PackPlan plan[3];
    std::vector<float> packed;           // all packed FP32 operators
    std::vector<int> off_cls;            // per M2L class
    std::vector<double> root_m2m, root_l2l, lattice;  // dense FP64 for the root
    std::vector<float> m2m_t, l2l_t;     // dense FP32, [octant][column][row], levels >= 1
    WorkPartition part[3];
    // tensor-core M2L (orders <= TC_MAX_ORDER): chunk plan and class images
    TcPlan tc;
    std::vector<uint8_t> tc_img;
};

// Row groups per contraction type: M2L has enough target tiles on its own;
// M2M and L2L split the output rows so that small levels still fill the GPU.
static const int k_groups[3] = {1, 4, 4};

std::mutex g_tab_mu;
std::vector<OpTables*> g_tabs;

const OpTables* get_tables(int P, int images)
{
    std::lock_guard<std::mutex> lk(g_tab_mu);
    for (OpTables* t : g_tabs)
        if (t->P == P && t->images == images) return t;
    OpTables* t = new OpTables();
    t->P = P;
    t->images = images;
    t->R = nreal(P);
    t->Rpad = (t->R + 3) & ~3;
    const int R = t->R;
    t->st = build_stencils(0.4);
    for (int k = 0; k < 3; k++) {
        t->plan[k] = make_pack_plan(P, (OpType)k);
        int g = k_groups[k];
        while (!make_work_items(t->plan[k], CT_WARPS, g, CT_MAXI, t->part[k])) g++;
    }
    std::vector<double> A((size_t)R * R);
    auto append = [&](const PackPlan& pl) {
        int off = (int)t->packed.size();
        t->packed.resize(t->packed.size() + pl.packed);
        pack_operator(pl, A.data(), t->packed.data() + off);
        return off;
    };
    // FP64 root operators in blocks of an even number of doubles (16-byte aligned
    // rows for bulk copies): M2M block o at o * R2p, the lattice padded to R2p
    const size_t R2p = ((size_t)R * R + 1) & ~(size_t)1;
    t->root_m2m.assign(8 * R2p, 0.0);
    t->root_l2l.resize((size_t)8 * R * R);
    t->m2m_t.assign((size_t)8 * R * R, 0.f);
    t->l2l_t.assign((size_t)8 * R * R, 0.f);
    auto transpose = [&](std::vector<float>& dst, int o) {
        for (int r = 0; r < R; r++)
            for (int c = 0; c < R; c++) dst[(size_t)o * R * R + (size_t)c * R + r] = (float)A[(size_t)r * R + c];
    };
    for (int o = 0; o < 8; o++) {
        scaled_m2m(P, o, A.data());
        std::copy(A.begin(), A.end(), t->root_m2m.begin() + o * R2p);
        transpose(t->m2m_t, o);
        scaled_l2l(P, o, A.data());
        std::copy(A.begin(), A.end(), t->root_l2l.begin() + (size_t)o * R * R);
        transpose(t->l2l_t, o);
    }
    t->off_cls.resize(t->st.classes.size());
    if (P <= TC_MAX_ORDER) t->tc = make_tc_plan(P);
    for (size_t c = 0; c < t->st.classes.size(); c++) {
        scaled_m2l(P, t->st.classes[c], A.data());
        t->off_cls[c] = append(t->plan[OP_M2L]);
        if (P <= TC_MAX_ORDER) append_tc_image(t->tc, R, A.data(), t->tc_img);
    }
    t->lattice.assign(R2p, 0.0);
    lattice_operator(P, images, t->lattice.data());
    g_tabs.push_back(t);
    return t;
}

}  // namespace

struct gbfmm_handle {
    gbfmm_params prm{};
    int n = 0, P = 0, R = 0, Rpad = 0, D = 0, nleaf = 0;
    bool periodic = true;
    // box shape: stored cells per axis of level l = grid_n(l, shift[d]); ncell[l]
    // stored cells of level l (8^l for a cube; a slab stores the box's quarter of
    // the root cube at every level >= 1)
    int aspect_z = 1;
    int shift[3] = {0, 0, 0};
    long ncell[MAX_DEPTH + 1] = {};
    const OpTables* tab = nullptr;
    cudaStream_t stream = nullptr;
    // P2P runs on its own low-priority stream, concurrently with the far field
    // (captured as a fork/join of the step graph)
    cudaStream_t stream_nf = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the deep levels' bf16 grids convert beside the upper-tree kernel
    cudaStream_t stream_g = nullptr;
    cudaEvent_t ev_gfork = nullptr, ev_gjoin = nullptr;
    // the tree-key node of the captured graph (its parameters carry the step's
    // constants) and the arguments it was captured with
    cudaGraph_t graph = nullptr;
    cudaGraphNode_t tk_node = nullptr;
    cudaKernelNodeParams tk_params = {};
    TreeArgs tk_args;
    StepConst tk_sc;  // the constants the node holds now
    // host state
    std::vector<float> h_q;
    bool have_charges = false, have_result = false, results_on_host = false;
    bool host_direct = false;       // the device reads pageable host memory: host calls work in place
    bool results_in_place = false;  // the last step wrote its results into the pinned host buffers
    int verbose = 0;
    // device arena
    void* arena = nullptr;
    size_t arena_bytes = 0;
    float* d_coords = nullptr;   // internal copy for host-side execute
    float* d_q = nullptr;
    uint32_t* d_code = nullptr;
    float4* d_uq = nullptr;
    int *d_counts = nullptr, *d_off = nullptr, *d_scan = nullptr, *d_tmp = nullptr;
    int *d_order = nullptr, *d_inv = nullptr;  // sorted -> input index, and its inverse
    int* d_leaf_edge = nullptr;                 // per leaf: a body on or near a face (the P2P r = 0 test)
    float4 *d_atoms = nullptr, *d_near = nullptr, *d_far = nullptr;
    float *d_M = nullptr, *d_L = nullptr;
    float* Mlev[8] = {};
    float* Llev[8] = {};
    size_t lev_floats = 0;
    double *d_M0 = nullptr, *d_L0 = nullptr;
    double* d_root_part = nullptr;  // 8 x R x 4 shares of the FP64 root M2M
    float* d_fconst = nullptr;      // dipole-correction constants of the finalize
    float* d_ops = nullptr;
    CEntry* d_entries = nullptr;
    size_t tasks_bytes = 0;  // entries + tasks allocation
    CTask* d_tasks = nullptr;
    int4* d_items[3] = {};
    int* d_wb[3] = {};
    BlockInfo* d_blocks[3] = {};
    double *d_root_m2m = nullptr, *d_root_l2l = nullptr, *d_lattice = nullptr;
    float *d_m2m_t = nullptr, *d_l2l_t = nullptr;

    int* d_p2p_st = nullptr;
    int n_p2p_st = 0;
    float *d_forces = nullptr, *d_pots = nullptr;
    double* d_energy = nullptr;
    double* d_sums = nullptr;
    double* d_partials = nullptr;
    int* d_flags = nullptr;
    // tensor-core M2L
    bool tc = false;
    __nv_bfloat16 *d_gh = nullptr, *d_gl = nullptr;  // tensor-core source grids (hi, lo)
    TcGrids tcg;
    TcArgs* tca = nullptr;  // tensor maps and launch arguments (host, 64-byte aligned)
    uint8_t* d_img = nullptr;
    CEntry* d_tc_entries = nullptr;
    // tensor-core M2L task lists, one per entry split 2^v (v < TC_NSPLIT)
    CTask* d_tc_tasks_v[TC_NSPLIT] = {};
    int tc_task0_v[TC_NSPLIT] = {}, tc_ntask_v[TC_NSPLIT] = {};
    int tc_split_v = 0;
    int tc_nstage = 2;
    int p2p_variant = 0;  // P2P warp-step shape (autotuned)
    int near_after = 0;   // the near field starts after the tree (0), the P2M (1) or the upper tree (2)
    bool pdl = true;      // consecutive kernels of the step's main chain launch as programmatic dependents
    StepConst* d_sc = nullptr;  // written by the tree-key kernel's block 0 each step
    StepConst* h_sc = nullptr;  // this step's constants (set_box), passed by value to that kernel
    int* h_flags = nullptr;     // pinned
    // task ranges
    int m2l_task0 = 0, m2l_ntask = 0;
    // graph
    cudaGraphExec_t gexec = nullptr;
    // host result staging (pinned)
    float* h_forces = nullptr;
    float* h_pots = nullptr;
    double* h_energy = nullptr;
    // stage timing
    bool timing = false;
    cudaEvent_t ev[16] = {};
    float stage_ms[16] = {};
    int n_stage = 0;
    int step_launches = 0;
    // virial pass (allocated on the first gbfmm_get_virial)
    void* vir_buf = nullptr;
    float* vir_lam = nullptr;         // 3 x lev_floats shift-weighted locals
    float4* vir_field = nullptr;      // 3 x N sorted fields of those locals
    double* vir_p2p = nullptr;        // 9 per leaf
    double* vir_out = nullptr;        // 27 per reduction block
    float* vir_ops = nullptr;         // dense transposed M2L operators per class
    CEntry* vir_entries = nullptr;    // M2L stencil entries, op = class index
    double* vir_lat = nullptr;        // 3 x R x R shift-weighted lattice operators
    int vir_e_first[2][8] = {}, vir_e_count[2][8] = {};
    int vir_blocks = 0;
};

static const char* k_stage_names[] = {"tree", "p2m", "m2m", "root", "m2l", "l2l", "l2p", "p2p", "finalize"};

extern "C" {

void gbfmm_params_default(gbfmm_params* p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->order = 10;
    p->max_depth = 3;
    p->images = 4;
    p->theta = 0.4;
    p->rega = 0.0;
    p->precision = GBFMM_PREC_FP32;
    p->aspect_z = 1;
}

const char* gbfmm_status_string(int s)
{
    switch (s) {
        case GBFMM_OK: return "ok";
        case GBFMM_ERR_ARG: return "invalid argument";
        case GBFMM_ERR_BOX: return "invalid box";
        case GBFMM_ERR_COORD: return "non-finite coordinate or charge";
        case GBFMM_ERR_CUDA: return "CUDA error";
        case GBFMM_ERR_NOMEM: return "out of memory";
        case GBFMM_ERR_UNSUPPORTED: return "unsupported";
        case GBFMM_ERR_STATE: return "call out of order";
        case GBFMM_ERR_TIMEOUT: return "device wait timed out";
        case GBFMM_ERR_NOT_NEUTRAL: return "system not neutral";
        default: return "unknown status";
    }
}

const char* gbfmm_last_error(void) { return g_err.c_str(); }
const char* gbfmm_version(void) { return "gbfmm 0.1 (sm_103a)"; }
const char* gbfmm_stage_name(int s) { return (s >= 0 && s < 9) ? k_stage_names[s] : ""; }

}  // extern "C"

// Destroys the step's graph (it is captured again on the next step).
static void drop_graph(gbfmm_handle* h)
{
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->gexec = nullptr;
    h->graph = nullptr;
    h->tk_node = nullptr;
}

static void free_handle(gbfmm_handle* h)
{
    if (!h) return;
    if (h->tca) {
        h->tca->~TcArgs();
        free(h->tca);
    }
    drop_graph(h);
    for (int i = 0; i < 16; i++)
        if (h->ev[i]) cudaEventDestroy(h->ev[i]);
    if (h->arena) cudaFree(h->arena);
    if (h->vir_buf) cudaFree(h->vir_buf);
    if (h->h_sc) cudaFreeHost(h->h_sc);
    if (h->h_flags) cudaFreeHost(h->h_flags);
    if (h->h_forces) cudaFreeHost(h->h_forces);
    if (h->h_pots) cudaFreeHost(h->h_pots);
    if (h->h_energy) cudaFreeHost(h->h_energy);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->stream_nf) cudaStreamDestroy(h->stream_nf);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->stream_g) cudaStreamDestroy(h->stream_g);
    if (h->ev_gfork) cudaEventDestroy(h->ev_gfork);
    if (h->ev_gjoin) cudaEventDestroy(h->ev_gjoin);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    delete h;
}

// Bump allocator over one device allocation.
struct Arena {
    size_t off = 0;
    char* base = nullptr;
    template <typename T>
    T* take(size_t count)
    {
        off = (off + 255) & ~(size_t)255;
        T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += sizeof(T) * count;
        return p;
    }
};

static int layout(gbfmm_handle* h, Arena& a)
{
    const int n = std::max(h->n, 1), R = h->R, Rpad = h->Rpad, D = h->D;
    const OpTables* t = h->tab;
    h->d_coords = a.take<float>(3 * (size_t)n);
    h->d_q = a.take<float>(n);
    h->d_code = a.take<uint32_t>(n);
    h->d_uq = a.take<float4>(n);
    h->d_counts = a.take<int>(h->nleaf + 1 + 4);  // + the epilogue counters (zeroed per step)
    h->d_off = a.take<int>(h->nleaf + 1);
    h->d_scan = a.take<int>((h->nleaf + 2047) / 2048 + 1);
    h->d_tmp = a.take<int>(n);
    h->d_order = a.take<int>(n);
    h->d_inv = a.take<int>(n);
    h->d_leaf_edge = a.take<int>(h->nleaf);
    h->d_atoms = a.take<float4>(n);
    h->d_near = a.take<float4>(n);
    h->d_far = a.take<float4>(n);
    size_t lev = 0;
    for (int k = 0; k <= D; k++) lev += (size_t)h->ncell[k] * Rpad;
    h->lev_floats = lev;
    h->d_M = a.take<float>(lev);
    h->d_L = a.take<float>(lev);
    if (h->tc) {
        h->tcg = tc_grid_layout(D, t->tc.k_atoms, h->shift);
        h->d_gh = a.take<__nv_bfloat16>((size_t)h->tcg.rows * h->tcg.KP);
        if (h->prm.precision != GBFMM_PREC_BF16X1) h->d_gl = a.take<__nv_bfloat16>((size_t)h->tcg.rows * h->tcg.KP);
        h->d_img = a.take<uint8_t>(t->tc_img.size());
    }
    h->d_M0 = a.take<double>(R);
    h->d_L0 = a.take<double>(R);
    h->d_root_part = a.take<double>(32 * (size_t)R);
    h->d_fconst = a.take<float>(4);
    h->d_ops = a.take<float>(t->packed.size());
    h->d_root_m2m = a.take<double>(t->root_m2m.size());
    h->d_root_l2l = a.take<double>(t->root_l2l.size());
    h->d_lattice = a.take<double>(t->lattice.size());
    h->d_m2m_t = a.take<float>(t->m2m_t.size());

    h->d_l2l_t = a.take<float>(t->l2l_t.size());
    h->d_p2p_st = a.take<int>(t->st.p2p.size());
    for (int k = 0; k < 3; k++) {
        h->d_items[k] = a.take<int4>(t->part[k].items.size() + 1);
        h->d_wb[k] = a.take<int>(t->part[k].warp_begin.size());
        h->d_blocks[k] = a.take<BlockInfo>(t->plan[k].nblk);
    }
    h->d_forces = a.take<float>(3 * (size_t)n);
    h->d_pots = a.take<float>(n);
    h->d_energy = a.take<double>(1);
    h->d_sums = a.take<double>(4);
    h->d_partials = a.take<double>(4 * std::max(TREE_MAX_BLOCKS, FINAL_MAX_BLOCKS));
    h->d_flags = a.take<int>(4);
    h->d_sc = a.take<StepConst>(1);
    return 0;
}

static void level_ptrs(gbfmm_handle* h)
{
    size_t o = 0;
    for (int k = 0; k <= h->D; k++) {
        h->Mlev[k] = h->d_M + o;
        h->Llev[k] = h->d_L + o;
        o += (size_t)h->ncell[k] * h->Rpad;
    }
}

// Task lists: the FP32 M2L contraction and the tensor-core M2L tiles.
static int build_tasks(gbfmm_handle* h)
{
    const OpTables* t = h->tab;
    const int D = h->D;
    std::vector<CEntry> ent;
    std::vector<CTask> tasks;
    // M2L stencils
    int e_m2l[2][8];
    for (int lt = 0; lt < 2; lt++)
        for (int s = 0; s < 8; s++) {
            e_m2l[lt][s] = (int)ent.size();
            for (const StencilEntry& se : t->st.m2l[lt][s]) {
                CEntry e;
                e.dx = (int8_t)se.d[0]; e.dy = (int8_t)se.d[1]; e.dz = (int8_t)se.d[2];
                e.mode = (int8_t)se.mode;
                e.op = t->off_cls[se.cls];
                ent.push_back(e);
            }
        }
    // M2L tasks (target octants of the stored grid only: a slab's level 1 holds
    // two of the root's eight octants)
    int split = h->prm.m2l_split > 0 ? h->prm.m2l_split : 1;
    if (h->prm.m2l_split <= 0) {
        long tiles = 0;
        for (int k = 1; k <= D; k++) tiles += 8 * std::max<long>(1, h->ncell[k - 1] / CT_TILE);
        while (tiles * split < 2 * sm_count() && split < 8) split *= 2;
    }
    if (h->prm.flags & GBFMM_FLAG_DETERMINISTIC) split = 1;
    h->m2l_task0 = (int)tasks.size();
    for (int k = 1; k <= D; k++) {
        const int lt = k == 1 ? 0 : 1;
        const long npar = h->ncell[k - 1];
        for (int s = 0; s < 8; s++) {
            if (!tc_octant_stored(k, h->shift, s)) continue;
            int eb = e_m2l[lt][s], ne = (int)t->st.m2l[lt][s].size();
            for (long q0 = 0; q0 < npar; q0 += CT_TILE) {
                int ch = (ne + split - 1) / split;
                const WorkPartition& wp = t->part[OP_M2L];
                for (int e0 = 0; e0 < ne; e0 += ch)
                    for (int g = 0; g < wp.groups; g++) {
                        CTask c;
                        c.level = k; c.octant = s; c.q0 = (int)q0; c.ntgt = (int)std::min<long>(CT_TILE, npar - q0);
                        c.e_begin = eb + e0; c.e_end = eb + std::min(ne, e0 + ch);
                        c.group = g; c.r0 = wp.row0[g]; c.r1 = wp.row1[g];
                        tasks.push_back(c);
                    }
            }
        }
    }
    h->m2l_ntask = (int)tasks.size() - h->m2l_task0;
    // tensor-core M2L: entries carry the class index, tiles of TC_TILE targets
    if (h->tc) {
        int e_tc[2][8];
        for (int lt = 0; lt < 2; lt++)
            for (int s = 0; s < 8; s++) {
                e_tc[lt][s] = (int)ent.size();
                for (const StencilEntry& se : t->st.m2l[lt][s]) {
                    CEntry e;
                    e.dx = (int8_t)se.d[0]; e.dy = (int8_t)se.d[1]; e.dz = (int8_t)se.d[2];
                    e.mode = (int8_t)se.mode;
                    e.op = se.cls;
                    ent.push_back(e);
                }
            }
        // task lists for the entry splits 1, 2, 4, 8 (a tile's stencil entries
        // cut into that many ranges; split > 1 adds into L with atomics); the
        // autotuner picks one, the default fills the GPU with CTAs
        long tiles = 0;
        for (int k = 1; k <= D; k++) tiles += 8L * tc_tiles(k, h->shift);
        int def = 0;
        if (h->prm.m2l_split > 0) {
            while (def < 3 && (1 << def) < h->prm.m2l_split) def++;
        } else {
            while (tiles * (1L << def) < sm_count() && def < 3) def++;
        }
        const bool det = (h->prm.flags & GBFMM_FLAG_DETERMINISTIC) != 0;
        if (det) def = 0;
        for (int v = 0; v < TC_NSPLIT; v++) {
            const int sp = 1 << v;
            h->tc_task0_v[v] = (int)tasks.size();
            if (det && v > 0) {
                h->tc_ntask_v[v] = 0;
                continue;
            }
            for (int k = 1; k <= D; k++) {
                const int lt = k == 1 ? 0 : 1;
                int bx, by, bz;
                tc_tile_shape(k, h->shift, bx, by, bz);
                for (int s = 0; s < 8; s++) {
                    if (!tc_octant_stored(k, h->shift, s)) continue;
                    int eb = e_tc[lt][s], ne = (int)t->st.m2l[lt][s].size();
                    int ch = (ne + sp - 1) / sp;
                    for (int q = 0; q < tc_tiles(k, h->shift); q++)
                        for (int e0 = 0; e0 < ne; e0 += ch) {
                            CTask c;
                            c.level = k; c.octant = s; c.q0 = q; c.ntgt = bx * by * bz;
                            c.e_begin = eb + e0; c.e_end = eb + std::min(ne, e0 + ch);
                            c.group = 0; c.r0 = 0; c.r1 = h->R;
                            tasks.push_back(c);
                        }
                }
            }
            h->tc_ntask_v[v] = (int)tasks.size() - h->tc_task0_v[v];
        }
        h->tc_split_v = def;
    }
    void* p = nullptr;
    h->tasks_bytes = sizeof(CEntry) * ent.size() + sizeof(CTask) * tasks.size() + 512;
    CK(cudaMalloc(&p, h->tasks_bytes));
    h->d_entries = (CEntry*)p;
    h->d_tasks = (CTask*)((char*)p + ((sizeof(CEntry) * ent.size() + 255) & ~(size_t)255));
    for (int v = 0; v < TC_NSPLIT; v++) h->d_tc_tasks_v[v] = h->d_tasks + h->tc_task0_v[v];
    CK(cudaMemcpy(h->d_entries, ent.data(), sizeof(CEntry) * ent.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->d_tasks, tasks.data(), sizeof(CTask) * tasks.size(), cudaMemcpyHostToDevice));
    return GBFMM_OK;
}

// Launch arguments of the tensor-core M2L, tensor maps included (encoded once:
// the grids do not move).
static int make_tc_args(gbfmm_handle* h)
{
    void* mem = nullptr;
    if (posix_memalign(&mem, 64, sizeof(TcArgs)) != 0) return fail(GBFMM_ERR_NOMEM, "host memory");
    TcArgs* a = new (mem) TcArgs();
    std::memset(a, 0, sizeof(TcArgs));
    h->tca = a;
    const TcPlan& pl = h->tab->tc;
    for (int d = 0; d < 3; d++) a->shift[d] = h->shift[d];
    a->leaf_off = h->d_off;
    a->depth = h->D;
    if (!tc_encode_maps(*a, h->D, h->tcg, h->d_gh, h->d_gl))
        return fail(GBFMM_ERR_CUDA, "tensor map encoding of the M2L source grids failed");
    for (int k = 0; k <= h->D; k++) a->dst_lvl[k] = h->Llev[k];
    a->bimg = h->d_img;
    a->entries = h->d_entries;
    a->tasks = h->d_tc_tasks_v[h->tc_split_v];
    a->err = h->d_flags + 1;
    a->wait_limit = WAIT_POLLS_DEFAULT;
    a->Rpad = h->Rpad;
    a->k_atoms = pl.k_atoms;
    a->img_bytes = pl.img_bytes;
    a->tmem_cols = pl.tmem_cols;
    a->nchunk = pl.nchunk;
    a->nprod = h->prm.precision == GBFMM_PREC_BF16X1 ? 1 : 3;
    a->group = TC_GROUP_DEFAULT;
    a->nstage = std::max(1, tc_pick_stages(pl.k_atoms, pl.img_bytes, a->nprod) / a->group);
    h->tc_nstage = a->nstage;
    if (tc_smem_bytes(*a) > 227 * 1024 - TC_MAXENT * sizeof(CEntry))
        return fail(GBFMM_ERR_UNSUPPORTED, "tensor-core M2L of order %d: one pipeline stage exceeds shared memory",
                    h->P);
    a->atomic = h->tc_split_v > 0 ? 1 : 0;
    for (int c = 0; c < pl.nchunk; c++) {
        a->chunk_n[c] = pl.n[c];
        a->chunk_k[c] = pl.k[c];
        a->chunk_col[c] = pl.col[c];
        a->chunk_row0[c] = pl.row0[c];
        a->chunk_rows[c] = pl.rows[c];
        a->chunk_img[c] = pl.img[c];
    }
    return GBFMM_OK;
}

static TcGridArgs tc_grid_args(gbfmm_handle* h)
{
    TcGridArgs g;
    const TcGrids& l = h->tcg;
    for (int k = 0; k <= h->D; k++) {
        if (k < h->D) {
            g.row0[g.ngrid] = l.n_row0[k];
            g.level[g.ngrid] = k;
            g.parity[g.ngrid] = 0;
            for (int d = 0; d < 3; d++) {
                g.W[g.ngrid][d] = l.n_w[k][d];
                g.n[g.ngrid][d] = grid_n(k, h->shift[d]);
            }
            g.src[g.ngrid++] = h->Mlev[k];
        }
        if (k >= 1) {
            g.row0[g.ngrid] = l.p_row0[k];
            g.level[g.ngrid] = k;
            g.parity[g.ngrid] = 1;
            for (int d = 0; d < 3; d++) {
                g.W[g.ngrid][d] = l.p_w[k][d];
                g.n[g.ngrid][d] = grid_n(k, h->shift[d]);
            }
            g.src[g.ngrid++] = h->Mlev[k];
        }
    }
    g.R = h->R;
    g.Rpad = h->Rpad;
    g.KP = l.KP;
    g.periodic = h->periodic ? 1 : 0;
    g.rows = l.rows;
    g.hi = h->d_gh;
    g.lo = h->d_gl;
    return g;
}

static ContractArgs contract_args(gbfmm_handle* h, int optype, int write_mode, bool src_is_L, int task0)
{
    ContractArgs a;
    std::memset(&a, 0, sizeof(a));
    a.ops = h->d_ops;
    a.entries = h->d_entries;
    a.tasks = h->d_tasks + task0;
    a.items = h->d_items[optype];
    a.warp_begin = h->d_wb[optype];
    a.blocks = h->d_blocks[optype];
    for (int k = 0; k <= h->D; k++) {
        a.src_lvl[k] = src_is_L ? h->Llev[k] : h->Mlev[k];
        a.dst_lvl[k] = optype == OP_M2M ? h->Mlev[k] : h->Llev[k];
    }
    a.R = h->R;
    a.Rpad = h->Rpad;
    a.nblk = h->tab->plan[optype].nblk;
    a.periodic = h->periodic ? 1 : 0;
    a.write_mode = write_mode;
    for (int d = 0; d < 3; d++) a.shift[d] = h->shift[d];
    a.leaf_off = optype == OP_M2L ? h->d_off : nullptr;
    a.depth = h->D;
    return a;
}

static void mark(gbfmm_handle* h, int stage)
{
    if (h->timing) cudaEventRecord(h->ev[stage], h->stream);
}

static P2PArgs p2p_args(const gbfmm_handle* h)
{
    P2PArgs pa;
    pa.off = h->d_off;
    pa.nleaf = h->nleaf;
    for (int d = 0; d < 3; d++) pa.nd[d] = grid_n(h->D, h->shift[d]);
    pa.periodic = h->periodic ? 1 : 0;
    pa.atoms = h->d_atoms;
    pa.stencil = h->d_p2p_st;
    pa.nst = h->n_p2p_st;
    pa.field = h->d_near;
    pa.leaf_edge = h->d_leaf_edge;
    pa.err = h->d_flags + 3;
    pa.wait_limit = WAIT_POLLS_DEFAULT;
    return pa;
}

// Phases of a step on h->stream: STEP_NEAR includes the near field (P2P), forked
// onto its own stream in graph mode; a batch leaves it out and runs all systems'
// near fields in one persistent kernel between the tree and the finalize.
enum { STEP_NEAR = 1, STEP_FINAL = 2 };

static void enqueue_final(gbfmm_handle* h);

// Enqueues one step on h->stream (captured into the graph on first use): the
// tree (tree_done, if given, is recorded after it), the near field (STEP_NEAR),
// the far field and the finalize (STEP_FINAL).
static void enqueue_step(gbfmm_handle* h, int mode = STEP_NEAR | STEP_FINAL, cudaEvent_t tree_done = nullptr)
{
    cudaStream_t s = h->stream;
    const int D = h->D, n = h->n;
    const long launches0 = g_kernel_launches.load();
    // a kernel that follows another on s without a cross-stream wait between them
    // starts as its programmatic dependent (off in the stage-timing pass, whose
    // events bracket each kernel)
    const bool pdl = h->pdl && !h->timing;
    mark(h, 0);
    // Leaf counts and the step's counters are zero when a step starts: zeroed at
    // creation, then re-zeroed by their last users (leaf sort, the last blocks of
    // the tree, upper-tree and finalize kernels) and after a reported device error.
    int* sync = h->d_counts + h->nleaf + 1;  // [0] tree keys, [1] finalize, [2] P2P queue, [3] upper tree
    {
        TreeArgs ta;
        ta.sc = nullptr;  // the constants travel with the launch (no copy node ahead of the tree)
        ta.sc_copy = h->d_sc;
        ta.charges = h->d_q;
        ta.n = n;
        ta.depth = D;
        ta.code = h->d_code;
        ta.uq = h->d_uq;
        ta.counts = h->d_counts;
        ta.rank = h->d_inv;  // arrival ranks, consumed by the scatter before the leaf sort writes inv
        ta.zero = reinterpret_cast<float4*>(h->d_L);  // lev_floats: levels of Rpad (a multiple of 4) floats
        ta.zero_n4 = (long)(h->lev_floats / 4);
        ta.partials = h->d_partials;
        ta.flags = h->d_flags;
        ta.done = sync;
        ta.sums = nullptr;  // summed by the upper-tree kernel, off the serial path
        if (h->nleaf <= TREE_EPILOGUE_MAX_LEAVES) {
            ta.off = h->d_off;
            ta.nleaf = h->nleaf;
        }
        // the small operators and lists of the later stages (the application's
        // other kernels evict them between steps)
        int k = 0;
        auto pf = [&](const void* p, size_t bytes) {
            if (p && bytes >= 16 && k < TreeArgs::MAX_PREFETCH) {
                ta.pf[k] = p;
                ta.pf_bytes[k++] = bytes;
            }
        };
        const OpTables* t = h->tab;
        pf(h->d_m2m_t, sizeof(float) * t->m2m_t.size());
        pf(h->d_root_m2m, (size_t)(reinterpret_cast<const char*>(h->d_lattice + t->lattice.size()) -
                                   reinterpret_cast<const char*>(h->d_root_m2m)));
        pf(h->d_l2l_t, sizeof(float) * t->l2l_t.size());
        pf(h->d_entries, h->tasks_bytes);
        pf(h->d_p2p_st, sizeof(int) * 3 * h->n_p2p_st);
        // the constants are a parameter of this launch: a captured graph gets them
        // updated on the node before each launch (run_step), from h->tk_args
        launch_tree_keys(ta, s, h->h_sc);
        h->tk_args = ta;
        if (!ta.off) launch_exclusive_scan(h->d_counts, h->d_off, h->nleaf, h->d_scan, s);
    }
    launch_scatter_ranked(h->d_code, n, h->d_off, h->d_inv, h->d_tmp, s, pdl);
    launch_leaf_sort(h->d_off, h->nleaf, h->d_tmp, h->d_uq, h->d_code, h->d_order, h->d_atoms, h->d_inv,
                     h->d_counts, s, h->d_leaf_edge, pdl);
    mark(h, 1);
    // The near field needs only the tree: in graph mode it forks onto its own
    // low-priority stream and overlaps the far-field chain below (joined before
    // finalize), from the tree on or from a later far-field kernel on
    // (h->near_after: 1 after the P2M, 2 after the upper tree), so that the
    // far-field kernels with large shared memory find SMs before the near field's
    // CTAs fill them; the stage-timing pass runs it in line, after L2P.
    const P2PArgs pa = p2p_args(h);
    const bool near = (mode & STEP_NEAR) != 0;
    const bool fork = near && !h->timing;
    if (tree_done) cudaEventRecord(tree_done, s);
    auto fork_near = [&](int point) {
        if (!fork || point != std::min(h->near_after, 2)) return;
        cudaEventRecord(h->ev_fork, s);
        cudaStreamWaitEvent(h->stream_nf, h->ev_fork, 0);
        launch_p2p(pa, h->p2p_variant, h->stream_nf, sync + 2);
        cudaEventRecord(h->ev_join, h->stream_nf);
    };
    fork_near(0);
    // upward pass: P2M with the M2M of the leaf parents in one launch, M2M launches
    // down to level 3, then levels 2 and 1 and the FP64 root in one launch (k_top)
    const bool fused = D >= 2 && launch_p2m_m2m(h->P, h->d_off, h->nleaf, h->d_atoms, h->Mlev[D], h->Mlev[D - 1],
                                                h->d_m2m_t, h->Rpad, s, pdl);
    if (!fused) launch_p2m(h->P, h->d_off, h->nleaf, h->d_atoms, h->Mlev[D], h->Rpad, s, pdl);
    fork_near(1);
    mark(h, 2);
    const int top_from = D == 1 || h->R > TOP_STAGE_MAX_R ? 1 : std::min(3, fused ? D - 1 : D);
    for (int k = fused ? D - 2 : D - 1; k >= top_from; k--)
        launch_m2m(h->Mlev[k + 1], h->Mlev[k], h->d_m2m_t, (int)h->ncell[k], h->R, h->Rpad, s, pdl);
    mark(h, 3);
    // the bf16 grids of the levels complete before the upper tree (from top_from
    // down; they are last in the grid buffers) convert on their own stream beside it
    const bool gfork = h->tc && !h->timing;
    long grid_split = 0;  // first row of those levels' grids
    if (h->tc) {
        const TcGridArgs all = tc_grid_args(h);
        grid_split = all.rows;
        for (int q = all.ngrid - 1; q >= 0 && all.level[q] >= top_from; q--) grid_split = all.row0[q];
    }
    if (gfork && grid_split < h->tcg.rows) {
        TcGridArgs deep = tc_grid_args(h);
        deep.row_begin = grid_split;
        cudaEventRecord(h->ev_gfork, s);
        cudaStreamWaitEvent(h->stream_g, h->ev_gfork, 0);
        launch_tc_grids(deep, h->stream_g);
        cudaEventRecord(h->ev_gjoin, h->stream_g);
    }
    RootArgs ra;
    ra.R = h->R;
    ra.Rpad = h->Rpad;
    ra.m2m = h->d_root_m2m;
    ra.l2l = h->d_root_l2l;
    ra.lattice = h->d_lattice;
    ra.M1 = h->Mlev[1];
    ra.M0 = h->d_M0;
    ra.L0 = h->d_L0;
    ra.M0f = h->Mlev[0];
    ra.L1 = h->Llev[1];
    ra.sc = h->d_sc;
    ra.images = h->prm.images;
    ra.n1 = (int)h->ncell[1];
    TopArgs top;
    top.root = ra;
    top.from = top_from;
    top.lattice = h->R <= TOP_LATTICE_MAX_R ? 1 : 0;
    top.Min = h->Mlev[top_from];
    top.M2 = D >= 2 ? h->Mlev[2] : nullptr;
    top.M1 = h->Mlev[1];
    top.m2m_t = h->d_m2m_t;
    top.part = h->d_root_part;
    top.tree_part = h->d_partials;
    top.tree_nblocks = tree_blocks(h->n);
    top.sums = h->d_sums;
    top.fconst = h->d_fconst;
    top.inv_natoms = 1.0 / std::max(h->n, 1);
    top.done = sync + 3;
    top.err = h->d_flags + 2;
    top.umask = (h->shift[0] == 0 ? 4 : 0) | (h->shift[1] == 0 ? 2 : 0) | (h->shift[2] == 0 ? 1 : 0);
    launch_top(top, s, pdl);
    fork_near(2);
    mark(h, 4);
    if (h->tc) {
        // the root L2L rides on the grid conversion, ahead of the M2L; the grids
        // of the upper levels (all of them in the stage-timing pass) convert here,
        // after the deep levels' conversion has joined (the M2L then follows this
        // launch alone, as its programmatic dependent)
        const bool gjoin = gfork && grid_split < h->tcg.rows;
        if (gjoin) cudaStreamWaitEvent(s, h->ev_gjoin, 0);
        TcGridArgs tg = tc_grid_args(h);
        if (gfork) tg.rows = grid_split;
        tg.root_l2l = h->d_root_l2l;
        tg.L0 = h->d_L0;
        tg.L1 = h->Llev[1];
        tg.root_R = h->R;
        tg.root_n1 = (int)h->ncell[1];
        launch_tc_grids(tg, s, pdl && !gjoin);
        TcArgs& ta = *h->tca;  // the current tuning: entry split and pipeline depth
        ta.tasks = h->d_tc_tasks_v[h->tc_split_v];
        ta.atomic = h->tc_split_v > 0 ? 1 : 0;
        ta.nstage = h->tc_nstage;
        launch_m2l_tc(ta, h->tc_ntask_v[h->tc_split_v], s, pdl);
    } else {
        ContractArgs a = contract_args(h, OP_M2L, 2, false, h->m2l_task0);
        launch_contract(a, h->m2l_ntask, s);
    }
    mark(h, 5);
    if (!h->tc) launch_root_l2l(ra, s);
    if (D >= 2) {
        // L2L of levels 2..D and L2P in one launch
        DownArgs da;
        da.nparent = (int)h->ncell[D - 1];
        da.off = h->d_off;
        da.atoms = h->d_atoms;
        for (int k = 0; k <= D; k++) da.L[k] = h->Llev[k];
        da.l2l_t = h->d_l2l_t;
        da.field = h->d_far;
        da.depth = D;
        da.Rpad = h->Rpad;
        da.err = h->d_flags + 2;
        da.wait_limit = WAIT_POLLS_DEFAULT;
        launch_down(h->P, da, s, pdl);
        mark(h, 6);
    } else {
        mark(h, 6);  // depth 1: the leaves are level 1, complete after the root L2L
        launch_l2p(h->P, h->d_off, h->nleaf, h->d_atoms, h->Llev[D], h->Rpad, h->d_far, s);
    }
    mark(h, 7);
    if (fork) cudaStreamWaitEvent(s, h->ev_join, 0);
    else if (near) launch_p2p(pa, h->p2p_variant, s, sync + 2);
    mark(h, 8);
    if (mode & STEP_FINAL) enqueue_final(h);
    mark(h, 9);
    h->step_launches = (int)(g_kernel_launches.load() - launches0);
}

// Forces, potentials and energy from the near and far fields (on h->stream).
static void enqueue_final(gbfmm_handle* h)
{
    cudaStream_t s = h->stream;
    const int n = h->n;
    int* sync = h->d_counts + h->nleaf + 1;
    if (n > 0) {
        FinalArgs fa;
        fa.sc = h->d_sc;
        fa.n = n;
        fa.atoms = h->d_atoms;
        fa.inv = h->d_inv;
        fa.near = h->d_near;
        fa.far = h->d_far;
        fa.fconst = h->d_fconst;
        fa.flags = h->d_flags;
        fa.partials = h->d_partials;
        fa.done = sync + 1;
        fa.zero_after = sync + 2;
        launch_finalize(fa, s);
    } else {
        cudaMemsetAsync(h->d_energy, 0, sizeof(double), s);
    }
}

extern "C" int gbfmm_create(const gbfmm_params* prm, int natoms, gbfmm_handle** out)
{
    if (!out) return fail(GBFMM_ERR_ARG, "out is NULL");
    *out = nullptr;
    gbfmm_params p;
    if (prm) p = *prm;
    else gbfmm_params_default(&p);
    if (natoms < 0) return fail(GBFMM_ERR_ARG, "natoms < 0");
    if (p.order < 2 || p.order > MAX_ORDER) return fail(GBFMM_ERR_ARG, "order %d outside [2,%d]", p.order, MAX_ORDER);
    if (p.max_depth < 1 || p.max_depth > MAX_DEPTH)
        return fail(GBFMM_ERR_ARG, "max_depth %d outside [1,%d]", p.max_depth, MAX_DEPTH);
    if (p.images < 0 || p.images > 8) return fail(GBFMM_ERR_ARG, "images %d outside [0,8]", p.images);
    if (std::fabs(p.theta - 0.4) > 1e-12)
        return fail(GBFMM_ERR_UNSUPPORTED, "theta %.6g: only the reference MAC scale 0.4 is supported", p.theta);
    if (p.rega != 0.0) return fail(GBFMM_ERR_UNSUPPORTED, "rega > 0 (regularised FMM) is not built");
    if (p.precision != GBFMM_PREC_FP32 && p.precision != GBFMM_PREC_BF16X3 && p.precision != GBFMM_PREC_BF16X1)
        return fail(GBFMM_ERR_ARG, "unknown precision %d", p.precision);
    if (p.precision != GBFMM_PREC_FP32 && p.order > TC_MAX_ORDER)
        return fail(GBFMM_ERR_UNSUPPORTED, "tensor-core M2L supports orders <= %d (got %d)", TC_MAX_ORDER, p.order);
    if (p.m2l_tile != 0 && p.m2l_tile != CT_TILE) return fail(GBFMM_ERR_ARG, "m2l_tile must be 0 or %d", CT_TILE);
    if (p.m2l_split < 0 || p.m2l_split > 16) return fail(GBFMM_ERR_ARG, "m2l_split outside [0,16]");
    if (p.aspect_z == 0) p.aspect_z = 1;
    if (p.aspect_z != 1 && p.aspect_z != 2)
        return fail(GBFMM_ERR_ARG, "aspect_z %d: 1 (cube) or 2 (slab, Lz = 2 Lx = 2 Ly)", p.aspect_z);
    if (p.aspect_z == 2 && p.images < 1)
        return fail(GBFMM_ERR_UNSUPPORTED, "a slab box is solved as periodic (images >= 1)");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return fail(GBFMM_ERR_CUDA, "no CUDA device available");
    }
    gbfmm_handle* h = new gbfmm_handle();
    h->prm = p;
    {
        int pageable = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
            cudaGetLastError();
            pageable = 0;
        }
        h->host_direct = pageable != 0 && !(p.flags & GBFMM_FLAG_HOST_COPY);
    }
    h->n = natoms;
    h->P = p.order;
    h->R = nreal(p.order);
    h->Rpad = (h->R + 3) & ~3;
    h->D = p.max_depth;
    h->aspect_z = p.aspect_z;
    if (p.aspect_z == 2) {
        h->shift[0] = h->shift[1] = 1;
        h->shift[2] = 0;
    }
    for (int k = 0; k <= h->D; k++) h->ncell[k] = grid_cells(k, h->shift);
    h->nleaf = (int)h->ncell[h->D];
    h->periodic = p.images > 0;
    h->tc = p.precision != GBFMM_PREC_FP32;
    h->tab = get_tables(h->P, p.images);
    h->h_q.assign(natoms, 0.0f);
    int rc = GBFMM_OK;
    auto bail = [&](int code) {
        free_handle(h);
        return code;
    };
    {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, hi) != cudaSuccess ||
            cudaStreamCreateWithPriority(&h->stream_nf, cudaStreamNonBlocking, lo) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess ||

            cudaStreamCreateWithPriority(&h->stream_g, cudaStreamNonBlocking, hi) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_gfork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_gjoin, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(GBFMM_ERR_CUDA, "stream create failed"));
    }
    Arena sz;
    layout(h, sz);
    h->arena_bytes = sz.off + 256;
    cudaError_t e = cudaMalloc(&h->arena, h->arena_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bail(fail(GBFMM_ERR_NOMEM, "device arena of %zu bytes: %s", h->arena_bytes, cudaGetErrorString(e)));
    }
    Arena ar;
    ar.base = (char*)h->arena;
    layout(h, ar);
    level_ptrs(h);
    const OpTables* t = h->tab;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (bytes && cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = GBFMM_ERR_CUDA;
    };
    up(h->d_ops, t->packed.data(), sizeof(float) * t->packed.size());
    up(h->d_root_m2m, t->root_m2m.data(), sizeof(double) * t->root_m2m.size());
    up(h->d_root_l2l, t->root_l2l.data(), sizeof(double) * t->root_l2l.size());
    up(h->d_lattice, t->lattice.data(), sizeof(double) * t->lattice.size());
    up(h->d_m2m_t, t->m2m_t.data(), sizeof(float) * t->m2m_t.size());
    up(h->d_l2l_t, t->l2l_t.data(), sizeof(float) * t->l2l_t.size());
    if (h->tc) up(h->d_img, t->tc_img.data(), t->tc_img.size());
    {
        // the P2P kernel stages the target leaf itself first (entry 0): only its
        // bodies can coincide with a target, so only they need the r = 0 test
        std::vector<int> st = t->st.p2p;
        for (size_t e = 0; e < st.size() / 3; e++)
            if (st[3 * e] == 0 && st[3 * e + 1] == 0 && st[3 * e + 2] == 0) {
                std::rotate(st.begin(), st.begin() + 3 * e, st.begin() + 3 * e + 3);
                break;
            }
        up(h->d_p2p_st, st.data(), sizeof(int) * st.size());
        h->n_p2p_st = (int)st.size() / 3;
    }
    for (int k = 0; k < 3; k++) {
        std::vector<int4> it;
        for (const WorkItem& w : t->part[k].items) it.push_back(make_int4(w.blk, w.ca, w.cb, 0));
        it.push_back(make_int4(0, 0, 0, 0));
        up(h->d_items[k], it.data(), sizeof(int4) * it.size());
        up(h->d_wb[k], t->part[k].warp_begin.data(), sizeof(int) * t->part[k].warp_begin.size());
        std::vector<BlockInfo> bi(t->plan[k].nblk);
        for (int b = 0; b < t->plan[k].nblk; b++) {
            bi[b].c0 = t->plan[k].c0[b];
            bi[b].off = t->plan[k].off[b];
        }
        up(h->d_blocks[k], bi.data(), sizeof(BlockInfo) * bi.size());
    }
    if (rc != GBFMM_OK) return bail(fail(rc, "operator upload failed"));
    cudaMemset(h->d_flags, 0, sizeof(int) * 4);
    cudaMemset(h->d_counts, 0, sizeof(int) * (h->nleaf + 1 + 4));  // then kept zero between steps
    cudaMemset(h->d_M, 0, sizeof(float) * h->lev_floats);
    rc = build_tasks(h);
    if (rc != GBFMM_OK) return bail(rc);
    if (h->tc) {
        rc = make_tc_args(h);
        if (rc != GBFMM_OK) return bail(rc);
    }
    if (cudaMallocHost(&h->h_sc, sizeof(StepConst)) != cudaSuccess ||
        cudaMallocHost(&h->h_flags, sizeof(int) * 4) != cudaSuccess ||
        cudaMallocHost(&h->h_forces, sizeof(float) * 3 * std::max(natoms, 1)) != cudaSuccess ||
        cudaMallocHost(&h->h_pots, sizeof(float) * std::max(natoms, 1)) != cudaSuccess ||
        cudaMallocHost(&h->h_energy, sizeof(double)) != cudaSuccess)
        return bail(fail(GBFMM_ERR_NOMEM, "pinned host buffers"));
    std::memset(h->h_sc, 0, sizeof(StepConst));
    for (int i = 0; i < 16; i++)
        if (cudaEventCreate(&h->ev[i]) != cudaSuccess) return bail(fail(GBFMM_ERR_CUDA, "event create"));
    *out = h;
    return GBFMM_OK;
}

extern "C" int gbfmm_destroy(gbfmm_handle* h)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->d_entries) cudaFree(h->d_entries);
    free_handle(h);
    return GBFMM_OK;
}

extern "C" int gbfmm_set_charges(gbfmm_handle* h, int natoms, const float* q)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (natoms != h->n) return fail(GBFMM_ERR_ARG, "natoms %d differs from the handle's %d", natoms, h->n);
    if (natoms > 0 && !q) return fail(GBFMM_ERR_ARG, "charges is NULL");
    for (int i = 0; i < natoms; i++)
        if (!std::isfinite(q[i])) return fail(GBFMM_ERR_COORD, "charge %d is not finite", i);
    std::memcpy(h->h_q.data(), q, sizeof(float) * natoms);
    CK(cudaMemcpyAsync(h->d_q, q, sizeof(float) * natoms, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->have_charges = true;
    return GBFMM_OK;
}

// Fills the box-dependent step constants.  A cubic box: the reference takes the
// period from box[XX][XX] and the root half-width as its half
// (zeta_fmm_solver.cpp:38-40).  A slab (aspect_z 2, Lx = Ly, Lz = 2 Lx): the root
// is the cube of edge Lz; the stored leaf grid covers the box itself, with cubic
// leaves of edge Lz / 2^D (2^(D-1) along x and y, 2^D along z), and the dipole
// correction takes the box's own volume.
// host_out: the finalize writes the results into the handle's pinned host
// buffers (a host call whose coordinates the device reads in place).
static int set_box(gbfmm_handle* h, const float* box, const float* d_coords, bool host_out = false)
{
    if (!box) return fail(GBFMM_ERR_ARG, "box is NULL");
    for (int i = 0; i < 9; i++)
        if (!std::isfinite(box[i])) return fail(GBFMM_ERR_BOX, "box entry %d is not finite", i);
    if (!(box[0] > 0) || box[1] != 0 || box[2] != 0 || box[3] != 0 || box[5] != 0 || box[6] != 0 || box[7] != 0)
        return fail(GBFMM_ERR_BOX, "box must be rectangular with positive diagonal");
    if (h->aspect_z == 1 && (box[4] != box[0] || box[8] != box[0]))
        return fail(GBFMM_ERR_BOX, "box must be cubic (got %g x %g x %g)", box[0], box[4], box[8]);
    if (h->aspect_z == 2 &&
        (box[4] != box[0] || std::fabs((double)box[8] - 2.0 * (double)box[0]) > 1e-6 * (double)box[8]))
        return fail(GBFMM_ERR_BOX, "slab box must have Lx = Ly and Lz = 2 Lx (got %g x %g x %g)", box[0], box[4],
                    box[8]);
    const double a = (double)box[0];
    const double C = h->aspect_z == 2 ? 2.0 * a : a;  // edge of the root cube
    const double E[3] = {a, a, C};                    // the box's extents
    const int D = h->D, nd = 1 << D;
    StepConst* sc = h->h_sc;
    sc->coords = d_coords;
    sc->out_forces = host_out ? h->h_forces : h->d_forces;
    sc->out_pots = host_out ? h->h_pots : h->d_pots;
    sc->out_energy = host_out ? h->h_energy : h->d_energy;
    sc->out_flags = host_out ? h->h_flags : nullptr;
    sc->inv_h = (float)(nd / C);
    sc->coef = 4.0 * M_PI / (3.0 * E[0] * E[1] * E[2]);
    sc->box_len = C;
    sc->inv_box_len = 1.0 / C;
    sc->copies = h->aspect_z == 2 ? 4 : 1;
    for (int d = 0; d < 3; d++) {
        const int n = grid_n(D, h->shift[d]);
        sc->nd[d] = n;
        sc->box_centre[d] = E[d] / 2;
        // leaf boundaries of the strict '>' descent: the descent around centre c with
        // half-width L/2 compares against c + L*(j/2^D - 1/2), exactly representable
        const double lo = E[d] / 2 - E[d] / 2;
        sc->thresh[d][0] = -INFINITY;
        for (int j = 1; j < n; j++) {
            double b = lo + E[d] * j / n;
            float f = (float)b;
            if ((double)f > b) f = std::nextafter(f, -INFINITY);
            sc->thresh[d][j] = f;
        }
        for (int j = n; j <= nd; j++) sc->thresh[d][j] = INFINITY;
        for (int j = 0; j < nd; j++) {
            double c = lo + E[d] * (2 * std::min(j, n - 1) + 1) / (2.0 * n);
            float hi = (float)c;
            float lo_f = (float)(c - (double)hi);
            sc->centre[d][j] = make_float2(hi, lo_f);
        }
    }
    return GBFMM_OK;
}

static bool graph_mode(const gbfmm_handle* h) { return !(h->prm.flags & GBFMM_FLAG_NO_GRAPH) && !h->timing; }

// One step (enqueue_step: its first kernel reads the step constants from the
// pinned host copy that set_box wrote).  In graph mode the graph is launched on
// 'launch' when on_launch is set (any stream, the legacy default stream 0
// included), else on the handle's stream.
static int run_step(gbfmm_handle* h, cudaStream_t launch = nullptr, bool on_launch = false)
{
    const bool use_graph = graph_mode(h);
    if (use_graph) {
        if (!h->gexec) {
            drop_graph(h);
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            enqueue_step(h);
            cudaError_t e = cudaStreamEndCapture(h->stream, &g);
            if (e != cudaSuccess) return fail(GBFMM_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&h->gexec, g, cudaGraphInstantiateFlagUseNodePriority);
            if (e != cudaSuccess) {
                cudaGraphDestroy(g);
                return fail(GBFMM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
            }
            h->graph = g;  // kept: its tree-key node is updated before each launch
            size_t nn = 0;
            CK(cudaGraphGetNodes(g, nullptr, &nn));
            std::vector<cudaGraphNode_t> nodes(nn);
            CK(cudaGraphGetNodes(g, nodes.data(), &nn));
            for (cudaGraphNode_t node : nodes) {
                cudaGraphNodeType type;
                cudaKernelNodeParams p;
                if (cudaGraphNodeGetType(node, &type) == cudaSuccess && type == cudaGraphNodeTypeKernel &&
                    cudaGraphKernelNodeGetParams(node, &p) == cudaSuccess && p.func == tree_keys_sc_kernel()) {
                    h->tk_node = node;
                    h->tk_params = p;
                    h->tk_sc = *h->h_sc;  // captured with these
                    break;
                }
            }
            if (!h->tk_node) {
                drop_graph(h);
                return fail(GBFMM_ERR_CUDA, "graph capture: no tree-key node");
            }
        } else if (std::memcmp(&h->tk_sc, h->h_sc, sizeof(StepConst)) != 0) {
            // this step's constants into the tree-key node (copied by the call),
            // unless the node holds them already (same box and coordinate array)
            void* args[2] = {&h->tk_args, h->h_sc};
            cudaKernelNodeParams p = h->tk_params;
            p.kernelParams = args;
            p.extra = nullptr;
            CK(cudaGraphExecKernelNodeSetParams(h->gexec, h->tk_node, &p));
            h->tk_sc = *h->h_sc;
        }
        CK(cudaGraphLaunch(h->gexec, on_launch ? launch : h->stream));
    } else {
        enqueue_step(h);
        CK(cudaGetLastError());
    }
    h->have_result = true;
    h->results_on_host = false;
    h->results_in_place = false;
    return GBFMM_OK;
}

extern "C" int gbfmm_execute_device(gbfmm_handle* h, const void* d_coords, const float* box, void* stream)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (!h->have_charges) return fail(GBFMM_ERR_STATE, "charges not set");
    if (h->n > 0 && !d_coords) return fail(GBFMM_ERR_ARG, "coordinates are NULL");
    int rc = set_box(h, box, (const float*)d_coords);
    if (rc) return rc;
    cudaStream_t us = (cudaStream_t)stream;
    cudaEvent_t ein = h->ev[14], eout = h->ev[15];
    if (graph_mode(h)) {
        // the step graph runs on the caller's stream, after any earlier work on
        // the handle's stream; later copies of the results follow it
        CK(cudaEventRecord(ein, h->stream));
        CK(cudaStreamWaitEvent(us, ein, 0));
        rc = run_step(h, us, true);
        if (rc) return rc;
        CK(cudaEventRecord(eout, us));
        CK(cudaStreamWaitEvent(h->stream, eout, 0));
        return GBFMM_OK;
    }
    // order the internal stream after the caller's stream, and the caller's after us
    CK(cudaEventRecord(ein, us));
    CK(cudaStreamWaitEvent(h->stream, ein, 0));
    rc = run_step(h);
    if (rc) return rc;
    CK(cudaEventRecord(eout, h->stream));
    CK(cudaStreamWaitEvent(us, eout, 0));
    return GBFMM_OK;
}

static int fetch(gbfmm_handle* h)
{
    if (!h->have_result) return fail(GBFMM_ERR_STATE, "no result: call gbfmm_execute first");
    if (h->results_on_host) return GBFMM_OK;
    const int n = h->n;
    if (!h->results_in_place) {
        CK(cudaMemcpyAsync(h->h_forces, h->d_forces, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(h->h_pots, h->d_pots, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(h->h_energy, h->d_energy, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(h->h_flags, h->d_flags, sizeof(int) * 4, cudaMemcpyDeviceToHost, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    if (h->timing) {
        h->n_stage = 9;
        for (int s = 0; s < 9; s++) cudaEventElapsedTime(&h->stage_ms[s], h->ev[s], h->ev[s + 1]);
    }
    h->results_on_host = true;
    if (h->h_flags[1] || h->h_flags[2] || h->h_flags[3]) {
        CK(cudaMemsetAsync(h->d_flags, 0, sizeof(int) * 4, h->stream));
        CK(cudaMemsetAsync(h->d_counts, 0, sizeof(int) * (h->nleaf + 1 + 4), h->stream));
        h->have_result = false;
        return fail(GBFMM_ERR_TIMEOUT, h->h_flags[1]   ? "a bounded device wait in the tensor-core M2L gave up"
                                       : h->h_flags[2] ? "a bounded device wait in the upper-tree or downward-pass kernel gave up"
                                                       : "a bounded device wait in the near-field kernel gave up");
    }
    if (h->h_flags[0]) {
        CK(cudaMemsetAsync(h->d_flags, 0, sizeof(int) * 4, h->stream));
        h->have_result = false;
        return fail(GBFMM_ERR_COORD, "non-finite coordinate or charge in the input");
    }
    return GBFMM_OK;
}

extern "C" int gbfmm_execute(gbfmm_handle* h, const float* coords, const float* box, int verbose)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (!h->have_charges) return fail(GBFMM_ERR_STATE, "charges not set");
    if (h->n > 0 && !coords) return fail(GBFMM_ERR_ARG, "coordinates are NULL");
    h->verbose = verbose;
    // Where the device reaches pageable host memory (NVLink-C2C on GB300), the
    // step reads the caller's coordinates in place and the finalize writes the
    // results into the pinned host buffers: no staging copies either way.
    const bool in_place = h->host_direct && h->n > 0;
    int rc = set_box(h, box, in_place ? coords : h->d_coords, in_place);
    if (rc) return rc;
    if (!in_place)
        CK(cudaMemcpyAsync(h->d_coords, coords, sizeof(float) * 3 * h->n, cudaMemcpyHostToDevice, h->stream));
    rc = run_step(h);
    if (rc) return rc;
    h->results_in_place = in_place;
    rc = fetch(h);
    if (rc == GBFMM_OK && verbose)
        std::printf("[gbfmm] natoms=%d P=%d depth=%d images=%d energy=%.8f\n", h->n, h->P, h->D, h->prm.images,
                    *h->h_energy);
    return rc;
}

// A device buffer larger than L2 (129 MB on GB300) written before each timed
// step of the autotuners; none when it cannot be allocated.
struct L2Flush {
    void* buf = nullptr;
    size_t bytes = 256u << 20;
    L2Flush()
    {
        if (cudaMalloc(&buf, bytes) != cudaSuccess) {
            cudaGetLastError();
            buf = nullptr;
        }
    }
    ~L2Flush()
    {
        if (buf) cudaFree(buf);
    }
    void run(cudaStream_t s) const
    {
        if (buf) cudaMemsetAsync(buf, 0, bytes, s);
    }
};

// ---- autotuner: warp-step shape of P2P, entry split and pipeline depth of the
// tensor-core M2L, chosen by timing whole steps (CUDA-graph replays) of the
// caller's own configuration.

static void apply_tuning(gbfmm_handle* h, int p2p_variant, int split_v, int nstage)
{
    h->p2p_variant = p2p_variant;
    h->tc_split_v = split_v;
    h->tc_nstage = nstage;
    drop_graph(h);
}

extern "C" int gbfmm_set_tuning(gbfmm_handle* h, int p2p_variant, int m2l_split, int m2l_stages)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (p2p_variant < 0 || p2p_variant >= p2p_variants()) return fail(GBFMM_ERR_ARG, "p2p variant %d", p2p_variant);
    int v = 0;
    while (v < TC_NSPLIT - 1 && (1 << v) < m2l_split) v++;
    if (m2l_split < 1 || (1 << v) != m2l_split) return fail(GBFMM_ERR_ARG, "m2l split %d is not 1, 2, 4 or 8", m2l_split);
    int ns = h->tc_nstage;
    if (h->tc) {
        if (h->tc_ntask_v[v] == 0) return fail(GBFMM_ERR_ARG, "m2l split %d unavailable (deterministic handle)", m2l_split);
        const TcPlan& pl = h->tab->tc;
        const int mx = std::max(1, tc_max_stages(pl.k_atoms, pl.img_bytes, h->tca->nprod) / h->tca->group);
        if (m2l_stages < 1 || m2l_stages > mx) return fail(GBFMM_ERR_ARG, "m2l stages %d outside [1,%d]", m2l_stages, mx);
        ns = m2l_stages;
    }
    CK(cudaStreamSynchronize(h->stream));
    apply_tuning(h, p2p_variant, v, ns);
    return GBFMM_OK;
}

extern "C" int gbfmm_set_near_start(gbfmm_handle* h, int after)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (after < 0 || after > 2) return fail(GBFMM_ERR_ARG, "near-field start %d outside [0,2]", after);
    CK(cudaStreamSynchronize(h->stream));
    h->near_after = after;
    drop_graph(h);
    return GBFMM_OK;
}

extern "C" int gbfmm_get_near_start(gbfmm_handle* h, int* after)
{
    if (!h || !after) return fail(GBFMM_ERR_ARG, "NULL argument");
    *after = h->near_after;
    return GBFMM_OK;
}

extern "C" int gbfmm_set_launch_overlap(gbfmm_handle* h, int enable)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    CK(cudaStreamSynchronize(h->stream));
    h->pdl = enable != 0;
    drop_graph(h);
    return GBFMM_OK;
}

extern "C" int gbfmm_get_launch_overlap(gbfmm_handle* h, int* enable)
{
    if (!h || !enable) return fail(GBFMM_ERR_ARG, "NULL argument");
    *enable = h->pdl ? 1 : 0;
    return GBFMM_OK;
}

extern "C" int gbfmm_get_tuning(gbfmm_handle* h, int* p2p_variant, int* m2l_split, int* m2l_stages)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (p2p_variant) *p2p_variant = h->p2p_variant;
    if (m2l_split) *m2l_split = 1 << h->tc_split_v;
    if (m2l_stages) *m2l_stages = h->tc_nstage;
    return GBFMM_OK;
}

extern "C" int gbfmm_autotune(gbfmm_handle* h, const float* coords, const float* box, int reps, float* best_ms)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (!h->have_charges) return fail(GBFMM_ERR_STATE, "charges not set");
    if (h->n > 0 && !coords) return fail(GBFMM_ERR_ARG, "coordinates are NULL");
    if (reps <= 0) reps = 5;
    int rc = set_box(h, box, h->d_coords);
    if (rc) return rc;
    CK(cudaMemcpyAsync(h->d_coords, coords, sizeof(float) * 3 * h->n, cudaMemcpyHostToDevice, h->stream));
    const bool timing = h->timing;
    h->timing = false;
    // each timed step starts from a flushed L2 (a write larger than L2 before it),
    // as steps do between which the application's other kernels run
    L2Flush flush;
    std::vector<cudaEvent_t> e0(reps), e1(reps);
    for (int i = 0; i < reps; i++) {
        CK(cudaEventCreate(&e0[i]));
        CK(cudaEventCreate(&e1[i]));
    }
    int err = GBFMM_OK;
    auto measure = [&](int pv, int sv, int ns) -> float {
        apply_tuning(h, pv, sv, ns);
        for (int i = 0; i < 2 && err == GBFMM_OK; i++) err = run_step(h);
        if (err) return 1e30f;
        for (int i = 0; i < reps && err == GBFMM_OK; i++) {
            flush.run(h->stream);
            cudaEventRecord(e0[i], h->stream);
            err = run_step(h);
            cudaEventRecord(e1[i], h->stream);
        }
        if (cudaEventSynchronize(e1[reps - 1]) != cudaSuccess) err = GBFMM_ERR_CUDA;
        float tot = 0.f;
        for (int i = 0; i < reps && !err; i++) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0[i], e1[i]);
            tot += ms;
        }
        return err ? 1e30f : tot / reps;
    };
    int bp = h->p2p_variant, bs = h->tc_split_v, bn = h->tc_nstage;
    float bt = measure(bp, bs, bn);
    auto search_p2p = [&]() {
        for (int pv = 0; pv < p2p_variants() && !err; pv++) {
            if (pv == bp) continue;
            const float t = measure(pv, bs, bn);
            if (t < bt) { bt = t; bp = pv; }
        }
    };
    // M2L entry split and pipeline depth together (each split with every depth
    // candidate: the best depth depends on how many CTAs the split makes)
    auto search_m2l = [&]() {
        if (!h->tc) return;
        const TcPlan& pl = h->tab->tc;
        const int gs = h->tca->group;
        const int mx = std::max(1, tc_max_stages(pl.k_atoms, pl.img_bytes, h->tca->nprod) / gs);
        // one stage: the most CTAs (and entries in flight) per SM
        const int cand[4] = {1, 2, std::max(1, tc_pick_stages(pl.k_atoms, pl.img_bytes, h->tca->nprod) / gs), mx};
        for (int sv = 0; sv < TC_NSPLIT && !err; sv++) {
            if (h->tc_ntask_v[sv] == 0) continue;
            for (int c = 0; c < 4 && !err; c++) {
                const int ns = std::min(cand[c], mx);
                if (ns < 1 || (sv == bs && ns == bn)) continue;
                bool dup = false;  // a depth already measured for this split
                for (int d = 0; d < c; d++) dup |= std::min(cand[d], mx) == ns;
                if (dup) continue;
                const float t = measure(bp, sv, ns);
                if (t < bt) { bt = t; bs = sv; bn = ns; }
            }
        }
    };
    // where the near field starts in the graph (after the tree, the P2M or the upper tree)
    auto search_near = [&]() {
        int ba = h->near_after;
        for (int na = 0; na <= 2 && !err; na++) {
            if (na == ba) continue;
            h->near_after = na;
            const float t = measure(bp, bs, bn);
            if (t < bt) { bt = t; ba = na; }
        }
        h->near_after = ba;
    };
    // coordinate search: P2P shape, the M2L (split x depth), the near field's start,
    // then the M2L and the P2P shape again at that start
    search_p2p();
    search_m2l();
    search_near();
    search_m2l();
    search_p2p();
    for (int i = 0; i < reps; i++) {
        cudaEventDestroy(e0[i]);
        cudaEventDestroy(e1[i]);
    }
    apply_tuning(h, bp, bs, bn);
    h->timing = timing;
    if (err) return err;
    if (best_ms) *best_ms = bt;
    return GBFMM_OK;
}

extern "C" int gbfmm_device_outputs(gbfmm_handle* h, void** f, void** p, void** e)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (f) *f = h->d_forces;
    if (p) *p = h->d_pots;
    if (e) *e = h->d_energy;
    return GBFMM_OK;
}

extern "C" int gbfmm_get_forces(gbfmm_handle* h, float* f)
{
    if (!h || (!f && h->n > 0)) return fail(GBFMM_ERR_ARG, "NULL argument");
    int rc = fetch(h);
    if (rc) return rc;
    std::memcpy(f, h->h_forces, sizeof(float) * 3 * h->n);
    return GBFMM_OK;
}

extern "C" int gbfmm_add_forces(gbfmm_handle* h, float* f)
{
    if (!h || (!f && h->n > 0)) return fail(GBFMM_ERR_ARG, "NULL argument");
    int rc = fetch(h);
    if (rc) return rc;
    for (int i = 0; i < 3 * h->n; i++) f[i] += h->h_forces[i];
    return GBFMM_OK;
}

extern "C" int gbfmm_get_potentials(gbfmm_handle* h, float* p)
{
    if (!h || (!p && h->n > 0)) return fail(GBFMM_ERR_ARG, "NULL argument");
    int rc = fetch(h);
    if (rc) return rc;
    std::memcpy(p, h->h_pots, sizeof(float) * h->n);
    return GBFMM_OK;
}

extern "C" int gbfmm_get_energy(gbfmm_handle* h, double* e)
{
    if (!h || !e) return fail(GBFMM_ERR_ARG, "NULL argument");
    int rc = fetch(h);
    if (rc) return rc;
    *e = *h->h_energy;
    return GBFMM_OK;
}

extern "C" int gbfmm_compare_forces(gbfmm_handle* h, const float* g, double* l2f)
{
    if (!h || !l2f || (!g && h->n > 0)) return fail(GBFMM_ERR_ARG, "NULL argument");
    int rc = fetch(h);
    if (rc) return rc;
    double dif = 0, nrm = 0;
    for (int i = 0; i < h->n; i++) {
        const float* f = h->h_forces + 3 * i;
        if (std::isnan(f[0]) || std::isnan(f[1]) || std::isnan(f[2]) || std::isnan(h->h_pots[i])) {
            *l2f = NAN;
            return fail(GBFMM_ERR_COORD, "result of atom %d is NaN", i);
        }
        for (int d = 0; d < 3; d++) {
            double x = (double)f[d] - (double)g[3 * i + d];
            dif += x * x;
            nrm += (double)g[3 * i + d] * (double)g[3 * i + d];
        }
    }
    *l2f = std::sqrt(dif / nrm);
    return GBFMM_OK;
}

extern "C" int gbfmm_step_launches(gbfmm_handle* h, int* n)
{
    if (!h || !n) return fail(GBFMM_ERR_ARG, "NULL argument");
    *n = h->step_launches;
    return GBFMM_OK;
}

extern "C" int gbfmm_set_timing(gbfmm_handle* h, int enable)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    h->timing = enable != 0;
    return GBFMM_OK;
}

extern "C" int gbfmm_stage_times(gbfmm_handle* h, float* ms, int n_max, int* n_out)
{
    if (!h || !ms || !n_out) return fail(GBFMM_ERR_ARG, "NULL argument");
    int rc = fetch(h);
    if (rc) return rc;
    int n = std::min(n_max, h->n_stage);
    for (int i = 0; i < n; i++) ms[i] = h->stage_ms[i];
    *n_out = n;
    return GBFMM_OK;
}

extern "C" int gbfmm_get_tree(gbfmm_handle* h, int* order, int* leaf_off, int* leaf_num)
{
    if (!h) return fail(GBFMM_ERR_ARG, "handle is NULL");
    if (!h->have_result) return fail(GBFMM_ERR_STATE, "no result: call gbfmm_execute first");
    std::vector<int> off(h->nleaf + 1);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(off.data(), h->d_off, sizeof(int) * (h->nleaf + 1), cudaMemcpyDeviceToHost));
    if (order) CK(cudaMemcpy(order, h->d_order, sizeof(int) * h->n, cudaMemcpyDeviceToHost));
    for (int k = 0; k < h->nleaf; k++) {
        if (leaf_off) leaf_off[k] = off[k];
        if (leaf_num) leaf_num[k] = off[k + 1] - off[k];
    }
    return GBFMM_OK;
}

extern "C" int gbfmm_lists(int max_depth, int images, int which, long* count, int* tgt, int* src, int* off3)
{
    if (!count || (which != 0 && which != 1) || max_depth < 1 || max_depth > MAX_DEPTH || images < 0 || images > 8)
        return fail(GBFMM_ERR_ARG, "bad argument");
    static std::mutex mu;
    static Stencils st;
    static bool have = false;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!have) {
            st = build_stencils(0.4);
            have = true;
        }
    }
    RefLists p2p, m2l;
    emit_lists(st, max_depth, images, p2p, m2l);
    const RefLists& l = which == 0 ? p2p : m2l;
    *count = (long)l.tgt.size();
    if (tgt) std::memcpy(tgt, l.tgt.data(), sizeof(int) * l.tgt.size());
    if (src) std::memcpy(src, l.src.data(), sizeof(int) * l.src.size());
    if (off3) std::memcpy(off3, l.off.data(), sizeof(int) * l.off.size());
    return GBFMM_OK;
}

extern "C" int gbfmm_get_lists(gbfmm_handle* h, int which, long* count, int* tgt, int* src, int* off3)
{
    if (!h || !count || (which != 0 && which != 1)) return fail(GBFMM_ERR_ARG, "bad argument");
    if (h->aspect_z != 1)
        return fail(GBFMM_ERR_UNSUPPORTED, "interaction lists in the reference's order exist for cubic boxes only");
    RefLists p2p, m2l;
    emit_lists(h->tab->st, h->D, h->prm.images, p2p, m2l);
    const RefLists& l = which == 0 ? p2p : m2l;
    *count = (long)l.tgt.size();
    if (tgt) std::memcpy(tgt, l.tgt.data(), sizeof(int) * l.tgt.size());
    if (src) std::memcpy(src, l.src.data(), sizeof(int) * l.src.size());
    if (off3) std::memcpy(off3, l.off.data(), sizeof(int) * l.off.size());
    return GBFMM_OK;
}

extern "C" int gbfmm_debug_operator(int order, int images, int kind, int index, double* mat, int* dim, double* cv)
{
    if (order < 2 || order > MAX_ORDER || !mat || !dim) return fail(GBFMM_ERR_ARG, "bad argument");
    const int R = nreal(order);
    *dim = R;
    if (kind == 0 || kind == 1) {
        if (index < 0 || index > 7) return fail(GBFMM_ERR_ARG, "octant %d", index);
        if (kind == 0) scaled_m2m(order, index, mat);
        else scaled_l2l(order, index, mat);
        return GBFMM_OK;
    }
    if (kind == 2) {
        Stencils st = build_stencils(0.4);
        if (index < 0 || index >= (int)st.classes.size()) return fail(GBFMM_ERR_ARG, "class %d", index);
        scaled_m2l(order, st.classes[index], mat);
        if (cv) {
            cv[0] = st.classes[index].kind;
            for (int i = 0; i < 3; i++) cv[1 + i] = st.classes[index].v[i];
        }
        return GBFMM_OK;
    }
    if (kind == 3) {
        lattice_operator(order, images, mat);
        return GBFMM_OK;
    }
    return fail(GBFMM_ERR_ARG, "kind %d", kind);
}

extern "C" int gbfmm_debug_bounded_wait(unsigned polls, void* stream)
{
    if (polls == 0) return fail(GBFMM_ERR_ARG, "polls must be positive");
    int* d_err = nullptr;
    CK(cudaMalloc(&d_err, sizeof(int)));
    cudaStream_t s = (cudaStream_t)stream;
    int flag = 0;
    cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(int), s);
    if (e == cudaSuccess) {
        launch_wait_probe(polls, d_err, s);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_err);
    if (e != cudaSuccess) return fail(GBFMM_ERR_CUDA, "bounded-wait probe: %s", cudaGetErrorString(e));
    if (flag) return fail(GBFMM_ERR_TIMEOUT, "the probe's bounded wait gave up after %u polls", polls);
    return GBFMM_OK;
}

extern "C" int gbfmm_debug_harmonics(int order, int kind, const double* d, double* out)
{
    if (order < 0 || order > 40 || !d || !out) return fail(GBFMM_ERR_ARG, "bad argument");
    int np = (order + 1) * (order + 2) / 2;
    std::vector<double> re(np), im(np);
    if (kind == 0) harm_regular(order, d, re.data(), im.data());
    else harm_singular(order, d, re.data(), im.data());
    for (int i = 0; i < np; i++) {
        out[2 * i] = re[i];
        out[2 * i + 1] = im[i];
    }
    return GBFMM_OK;
}

// ---- virial of the last step (virial.cu): Xi = -1/2 sum_i r_i (x) F_i + G / 4 plus
// the tin-foil term, G the image-shift-weighted forces of the interactions that
// cross the box (near-field and M2L stencil entries that wrap, far lattice).

static int virial_setup(gbfmm_handle* h)
{
    const OpTables* t = h->tab;
    const int R = h->R, ncls = (int)t->st.classes.size();
    std::vector<CEntry> ent;
    for (int lt = 0; lt < 2; lt++)
        for (int s = 0; s < 8; s++) {
            h->vir_e_first[lt][s] = (int)ent.size();
            for (const StencilEntry& se : t->st.m2l[lt][s]) {
                CEntry e;
                e.dx = (int8_t)se.d[0]; e.dy = (int8_t)se.d[1]; e.dz = (int8_t)se.d[2];
                e.mode = (int8_t)se.mode;
                e.op = se.cls;
                ent.push_back(e);
            }
            h->vir_e_count[lt][s] = (int)ent.size() - h->vir_e_first[lt][s];
        }
    std::vector<float> ops((size_t)ncls * R * R);
    std::vector<double> A((size_t)R * R);
    for (int c = 0; c < ncls; c++) {
        scaled_m2l(h->P, t->st.classes[c], A.data());
        for (int r = 0; r < R; r++)
            for (int col = 0; col < R; col++) ops[(size_t)c * R * R + (size_t)col * R + r] = (float)A[(size_t)r * R + col];
    }
    std::vector<double> lat(3 * (size_t)R * R);
    lattice_shift_operators(h->P, h->prm.images, lat.data());
    h->vir_blocks = std::max(1, std::min(4 * sm_count(), h->nleaf));
    Arena sz;
    for (int pass = 0; pass < 2; pass++) {
        Arena a;
        a.base = pass ? (char*)h->vir_buf : nullptr;
        h->vir_lam = a.take<float>(3 * h->lev_floats);
        h->vir_field = a.take<float4>(3 * (size_t)std::max(h->n, 1));
        h->vir_p2p = a.take<double>(9 * (size_t)h->nleaf);
        h->vir_out = a.take<double>(27 * (size_t)h->vir_blocks);
        h->vir_ops = a.take<float>(ops.size());
        h->vir_entries = a.take<CEntry>(ent.size());
        h->vir_lat = a.take<double>(lat.size());
        if (pass == 0) {
            cudaError_t e = cudaMalloc(&h->vir_buf, a.off + 256);
            if (e != cudaSuccess) {
                cudaGetLastError();
                h->vir_buf = nullptr;
                return fail(GBFMM_ERR_NOMEM, "virial buffers: %s", cudaGetErrorString(e));
            }
        }
    }
    CK(cudaMemcpy(h->vir_ops, ops.data(), sizeof(float) * ops.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->vir_entries, ent.data(), sizeof(CEntry) * ent.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->vir_lat, lat.data(), sizeof(double) * lat.size(), cudaMemcpyHostToDevice));
    return GBFMM_OK;
}

extern "C" int gbfmm_get_virial(gbfmm_handle* h, double* vir)
{
    if (!h || !vir) return fail(GBFMM_ERR_ARG, "NULL argument");
    if (!h->have_result) return fail(GBFMM_ERR_STATE, "no result: call gbfmm_execute first");
    if (h->P > 16 || h->R > VIR_MAXR) return fail(GBFMM_ERR_UNSUPPORTED, "virial: order %d", h->P);
    int rc = fetch(h);  // the step has completed without an error
    if (rc) return rc;
    if (!h->vir_buf) {
        rc = virial_setup(h);
        if (rc) return rc;
    }
    cudaStream_t s = h->stream;
    const int D = h->D;
    CK(cudaMemsetAsync(h->vir_lam, 0, sizeof(float) * 3 * h->lev_floats, s));
    float* lam[3][MAX_DEPTH + 1] = {};
    for (int x = 0; x < 3; x++) {
        size_t o = 0;
        for (int k = 0; k <= D; k++) {
            lam[x][k] = h->vir_lam + x * h->lev_floats + o;
            o += (size_t)h->ncell[k] * h->Rpad;
        }
    }
    // near field: the wrapped stencil entries
    P2PArgs pa = p2p_args(h);
    launch_virial_p2p(pa, h->vir_p2p, s);
    // M2L: the wrapped entries into the shift-weighted locals
    if (h->periodic) {
        VirialM2LArgs va;
        std::memset(&va, 0, sizeof(va));
        va.depth = D;
        va.R = h->R;
        va.Rpad = h->Rpad;
        for (int k = 0; k <= D; k++) va.ncell[k] = h->ncell[k];
        for (int d = 0; d < 3; d++) va.shift[d] = h->shift[d];
        va.entries = h->vir_entries;
        std::memcpy(va.e_first, h->vir_e_first, sizeof(va.e_first));
        std::memcpy(va.e_count, h->vir_e_count, sizeof(va.e_count));
        va.ops = h->vir_ops;
        for (int k = 0; k <= D; k++) va.M[k] = h->Mlev[k];
        for (int x = 0; x < 3; x++)
            for (int k = 0; k <= D; k++) va.lam[x][k] = lam[x][k];
        launch_virial_m2l(va, s);
    }
    // far lattice images, weighted by their index, at the root and L2L to level 1
    const double a_edge = (double)h->h_sc->box_len / (h->aspect_z == 2 ? 2.0 : 1.0);
    const double E[3] = {a_edge, a_edge, (double)h->h_sc->box_len};  // the box's periods
    if (h->prm.images >= 2) {
        VirialRootArgs ra;
        ra.R = h->R;
        ra.Rpad = h->Rpad;
        ra.n1 = (int)h->ncell[1];
        ra.lat_shift = h->vir_lat;
        ra.M0 = h->d_M0;
        ra.l2l = h->d_root_l2l;
        for (int x = 0; x < 3; x++) {
            ra.scale[x] = (double)h->h_sc->box_len / E[x];  // root-cube images in periods of the box
            ra.lam1[x] = lam[x][1];
        }
        launch_virial_root(ra, s);
    }
    // downward pass of each shift-weighted local to the bodies
    for (int x = 0; x < 3; x++) {
        float4* field = h->vir_field + (size_t)x * std::max(h->n, 1);
        if (D >= 2) {
            DownArgs da;
            da.nparent = (int)h->ncell[D - 1];
            da.off = h->d_off;
            da.atoms = h->d_atoms;
            for (int k = 0; k <= D; k++) da.L[k] = lam[x][k];
            da.l2l_t = h->d_l2l_t;
            da.field = field;
            da.depth = D;
            da.Rpad = h->Rpad;
            da.err = h->d_flags + 2;
            da.wait_limit = WAIT_POLLS_DEFAULT;
            launch_down(h->P, da, s);
        } else {
            launch_l2p(h->P, h->d_off, h->nleaf, h->d_atoms, lam[x][1], h->Rpad, field, s);
        }
    }
    VirialReduceArgs rd;
    rd.sc = h->d_sc;
    rd.nleaf = h->nleaf;
    rd.off = h->d_off;
    rd.atoms = h->d_atoms;
    rd.near = h->d_near;
    rd.far = h->d_far;
    for (int x = 0; x < 3; x++) rd.lam_field[x] = h->vir_field + (size_t)x * std::max(h->n, 1);
    rd.p2p_part = h->vir_p2p;
    rd.out = h->vir_out;
    launch_virial_reduce(rd, h->vir_blocks, s);
    CK(cudaGetLastError());
    std::vector<double> out(27 * (size_t)h->vir_blocks);
    double sums[4];
    CK(cudaMemcpyAsync(out.data(), h->vir_out, sizeof(double) * out.size(), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(sums, h->d_sums, sizeof(sums), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    double W[9] = {}, Gf[9] = {}, Gp[9] = {};
    for (int b = 0; b < h->vir_blocks; b++)
        for (int c = 0; c < 9; c++) {
            W[c] += out[27 * (size_t)b + c];
            Gf[c] += out[27 * (size_t)b + 9 + c];
            Gp[c] += out[27 * (size_t)b + 18 + c];
        }
    const double inv_h = (double)h->h_sc->inv_h, kp = KE * inv_h * inv_h;
    const double V = E[0] * E[1] * E[2];
    const double M[3] = {sums[0], sums[1], sums[2]}, M2 = M[0] * M[0] + M[1] * M[1] + M[2] * M[2];
    for (int x = 0; x < 3; x++)
        for (int y = 0; y < 3; y++) {
            const double G = h->periodic ? E[x] * (Gf[3 * x + y] + kp * Gp[3 * x + y]) : 0.0;
            const double corr = -M_PI * KE / (3.0 * V) * (2.0 * M[x] * M[y] - (x == y ? M2 : 0.0));
            vir[3 * x + y] = -0.5 * W[3 * x + y] + 0.25 * G + corr;
        }
    return GBFMM_OK;
}

// ---- batched solves
//
// Many independent cubic systems solved together: each system keeps its own
// operator set, stencils and tree (its own order and depth), but its inputs and
// outputs are views into packed batch buffers and all systems' steps are captured
// into ONE CUDA graph, forked over several streams so that independent systems
// run concurrently.  Per call the host uploads the step constants of every system
// in one copy and replays the graph.
struct gbfmm_batch {
    int n_sys = 0;
    long natoms = 0;
    std::vector<int> off;
    std::vector<gbfmm_handle*> hs;
    void* buf = nullptr;
    float *d_coords = nullptr, *d_q = nullptr, *d_forces = nullptr, *d_pots = nullptr;
    double* d_energy = nullptr;
    StepConst* d_sc = nullptr;
    StepConst* h_sc = nullptr;  // pinned
    cudaStream_t master = nullptr;
    std::vector<cudaStream_t> workers;
    std::vector<cudaEvent_t> ev;
    cudaEvent_t ein = nullptr, eout = nullptr;
    cudaEvent_t ev_sc = nullptr;  // the copy of h_sc has been made
    cudaGraphExec_t gexec = nullptr;
    bool have_result = false;
    // the systems' near fields in one persistent kernel
    void* p2p_buf = nullptr;  // P2PArgs[n_sys], first[n_sys+1], counter
    P2PBatchArgs p2p{};
    int p2p_shape = 0, p2p_per_sm = 4;  // near-field kernel shape and CTAs per SM (batch autotuner)
    int m2l_split_v = -1, m2l_stages = 0;  // batch-wide M2L tuning of the tensor-core systems (-1 / 0: their own)
    cudaStream_t near_stream = nullptr;
    std::vector<cudaEvent_t> ev_tree;
    cudaEvent_t ev_near = nullptr;
    // argument tables of the grouped launches (rebuilt at each capture)
    void* group_buf = nullptr;
    size_t group_bytes = 0;
    int step_launches = 0;  // kernels one batch step launches
    // Far-field lanes: the systems' far chains split by expansion order over
    // 'far_lanes' streams (workers, or workers_hi at the greatest stream priority
    // when far_prio), and the point at which the near-field kernel starts
    // (near_after 0: after the tree; 1: with the M2L; 2: after the M2L).
    std::vector<cudaStream_t> workers_hi;
    std::vector<cudaEvent_t> ev_up;
    int far_lanes = 1, near_after = 0;
    bool far_prio = false;
};

static void free_batch(gbfmm_batch* b)
{
    if (!b) return;
    for (gbfmm_handle* h : b->hs)
        if (h) gbfmm_destroy(h);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (cudaStream_t s : b->workers) cudaStreamDestroy(s);
    for (cudaStream_t s : b->workers_hi) cudaStreamDestroy(s);
    for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
    for (cudaEvent_t e : b->ev_up) cudaEventDestroy(e);
    if (b->ein) cudaEventDestroy(b->ein);
    if (b->ev_sc) cudaEventDestroy(b->ev_sc);
    if (b->eout) cudaEventDestroy(b->eout);
    if (b->master) cudaStreamDestroy(b->master);
    if (b->buf) cudaFree(b->buf);
    if (b->h_sc) cudaFreeHost(b->h_sc);
    if (b->p2p_buf) cudaFree(b->p2p_buf);
    if (b->group_buf) cudaFree(b->group_buf);
    if (b->near_stream) cudaStreamDestroy(b->near_stream);
    for (cudaEvent_t e : b->ev_tree) cudaEventDestroy(e);
    if (b->ev_near) cudaEventDestroy(b->ev_near);
    delete b;
}

static int batch_create(int n_sys, const int* atom_offsets, const int* orders, const int* depths,
                        const int* precisions, int precision, int images, int flags, gbfmm_batch** out);

extern "C" int gbfmm_batch_create(int n_sys, const int* atom_offsets, const int* orders, const int* depths, int images,
                                  int precision, int flags, gbfmm_batch** out)
{
    return batch_create(n_sys, atom_offsets, orders, depths, nullptr, precision, images, flags, out);
}

extern "C" int gbfmm_batch_create_mixed(int n_sys, const int* atom_offsets, const int* orders, const int* depths,
                                        const int* precisions, int images, int flags, gbfmm_batch** out)
{
    if (!precisions) return fail(GBFMM_ERR_ARG, "precisions is NULL");
    return batch_create(n_sys, atom_offsets, orders, depths, precisions, 0, images, flags, out);
}

static int batch_create(int n_sys, const int* atom_offsets, const int* orders, const int* depths,
                        const int* precisions, int precision, int images, int flags, gbfmm_batch** out)
{
    if (!out) return fail(GBFMM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n_sys <= 0 || !atom_offsets || !orders || !depths) return fail(GBFMM_ERR_ARG, "bad batch description");
    if (atom_offsets[0] != 0) return fail(GBFMM_ERR_ARG, "atom_offsets[0] must be 0");
    for (int i = 0; i < n_sys; i++)
        if (atom_offsets[i + 1] < atom_offsets[i]) return fail(GBFMM_ERR_ARG, "atom_offsets must not decrease");
    gbfmm_batch* b = new gbfmm_batch();
    b->n_sys = n_sys;
    b->off.assign(atom_offsets, atom_offsets + n_sys + 1);
    b->natoms = atom_offsets[n_sys];
    const size_t N = (size_t)std::max<long>(b->natoms, 1);
    auto bail = [&](int rc) {
        free_batch(b);
        return rc;
    };
    Arena sz;
    sz.take<float>(3 * N);
    sz.take<float>(N);
    sz.take<float>(3 * N);
    sz.take<float>(N);
    sz.take<double>(n_sys);
    sz.take<StepConst>(n_sys);
    if (cudaMalloc(&b->buf, sz.off + 256) != cudaSuccess) {
        cudaGetLastError();
        return bail(fail(GBFMM_ERR_NOMEM, "batch buffers"));
    }
    Arena ar;
    ar.base = (char*)b->buf;
    b->d_coords = ar.take<float>(3 * N);
    b->d_q = ar.take<float>(N);
    b->d_forces = ar.take<float>(3 * N);
    b->d_pots = ar.take<float>(N);
    b->d_energy = ar.take<double>(n_sys);
    b->d_sc = ar.take<StepConst>(n_sys);
    if (cudaMallocHost(&b->h_sc, sizeof(StepConst) * n_sys) != cudaSuccess) return bail(fail(GBFMM_ERR_NOMEM, "pinned"));
    std::memset(b->h_sc, 0, sizeof(StepConst) * n_sys);
    for (int i = 0; i < n_sys; i++) {
        gbfmm_params p;
        gbfmm_params_default(&p);
        p.order = orders[i];
        p.max_depth = depths[i];
        p.images = images;
        p.precision = precisions ? precisions[i] : precision;
        p.flags = flags & ~GBFMM_FLAG_NO_GRAPH;
        gbfmm_handle* h = nullptr;
        int rc = gbfmm_create(&p, atom_offsets[i + 1] - atom_offsets[i], &h);
        if (rc != GBFMM_OK) return bail(rc);
        b->hs.push_back(h);
        // the system's inputs and outputs are views of the batch buffers
        const int o = atom_offsets[i];
        h->d_q = b->d_q + o;
        h->d_forces = b->d_forces + 3 * (size_t)o;
        h->d_pots = b->d_pots + o;
        h->d_energy = b->d_energy + i;
        h->d_sc = b->d_sc + i;
        h->have_charges = true;
    }
    const int nw = std::min(n_sys, 8);
    if (cudaStreamCreateWithFlags(&b->master, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(GBFMM_ERR_CUDA, "stream create"));
    for (int w = 0; w < nw; w++) {
        cudaStream_t s;
        cudaEvent_t e;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(GBFMM_ERR_CUDA, "stream create"));
        b->workers.push_back(s);
        b->ev.push_back(e);
    }
    {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        for (int w = 0; w < nw; w++) {
            cudaStream_t s;
            cudaEvent_t e;
            if (cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, greatest) != cudaSuccess ||
                cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                return bail(fail(GBFMM_ERR_CUDA, "stream create"));
            b->workers_hi.push_back(s);
            b->ev_up.push_back(e);
        }
    }
    if (cudaEventCreateWithFlags(&b->ein, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_sc, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->eout, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_near, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(GBFMM_ERR_CUDA, "event create"));
    {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (cudaStreamCreateWithPriority(&b->near_stream, cudaStreamNonBlocking, lo) != cudaSuccess)
            return bail(fail(GBFMM_ERR_CUDA, "stream create"));
    }
    for (int i = 0; i < n_sys; i++) {
        cudaEvent_t e;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(GBFMM_ERR_CUDA, "event create"));
        b->ev_tree.push_back(e);
    }
    // near-field queue: systems ordered by bodies per leaf, heaviest first
    {
        std::vector<int> ord(n_sys);
        for (int i = 0; i < n_sys; i++) ord[i] = i;
        auto per_leaf = [&](int i) { return (double)b->hs[i]->n / (double)b->hs[i]->nleaf; };
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return per_leaf(x) > per_leaf(y); });
        std::vector<P2PArgs> args(n_sys);
        std::vector<int> first(n_sys + 1, 0);
        for (int k = 0; k < n_sys; k++) {
            args[k] = p2p_args(b->hs[ord[k]]);
            first[k + 1] = first[k] + b->hs[ord[k]]->nleaf;
        }
        const size_t a_b = (sizeof(P2PArgs) * n_sys + 255) & ~(size_t)255;
        const size_t f_b = (sizeof(int) * (n_sys + 1) + 255) & ~(size_t)255;
        if (cudaMalloc(&b->p2p_buf, a_b + f_b + 256) != cudaSuccess) {
            cudaGetLastError();
            return bail(fail(GBFMM_ERR_NOMEM, "batch queue"));
        }
        char* base = (char*)b->p2p_buf;
        if (cudaMemcpy(base, args.data(), sizeof(P2PArgs) * n_sys, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(base + a_b, first.data(), sizeof(int) * (n_sys + 1), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(GBFMM_ERR_CUDA, "batch queue upload"));
        b->p2p.sys = (const P2PArgs*)base;
        b->p2p.first = (const int*)(base + a_b);
        b->p2p.nsys = n_sys;
        b->p2p.nitems = first[n_sys];
        b->p2p.counter = (int*)(base + a_b + f_b);
    }
    *out = b;
    return GBFMM_OK;
}

// One system's step as launch descriptions: the arguments and grid sizes of the
// kernels enqueue_step launches for it, in the same order and with the same
// arithmetic (the batch runs each kind of kernel for all systems in one launch).
struct StepDesc {
    gbfmm_handle* h = nullptr;
    TreeArgs tree;
    int tree_blocks = 0;
    size_t tree_smem = 0;
    ScatterArgs scatter{};
    int scatter_blocks = 0;
    LeafSortArgs leaf{};
    int leaf_blocks = 0;
    bool fused = false;
    P2MArgs p2m{};
    int p2m_blocks = 0;
    std::vector<M2MArgs> m2m;  // levels from the finest up
    TopArgs top;
    size_t top_smem = 0;
    bool top_staged = false;
    RootArgs root{};
    TcGridArgs grids;
    int grids_blocks = 0;
    int m2l_blocks = 0;
    size_t m2l_smem = 0;
    DownArgs down{};
    L2PArgs l2p{};
    FinalArgs fin;
    int fin_blocks = 0;
};

static void describe_step(gbfmm_handle* h, StepDesc& d)
{
    const int D = h->D, n = h->n;
    d.h = h;
    int* sync = h->d_counts + h->nleaf + 1;
    TreeArgs& ta = d.tree;
    ta.sc = h->d_sc;
    ta.charges = h->d_q;
    ta.n = n;
    ta.depth = D;
    ta.code = h->d_code;
    ta.uq = h->d_uq;
    ta.counts = h->d_counts;
    ta.rank = h->d_inv;
    ta.zero = reinterpret_cast<float4*>(h->d_L);
    ta.zero_n4 = (long)(h->lev_floats / 4);
    ta.partials = h->d_partials;
    ta.flags = h->d_flags;
    ta.done = sync;
    ta.sums = nullptr;
    if (h->nleaf <= TREE_EPILOGUE_MAX_LEAVES) {
        ta.off = h->d_off;
        ta.nleaf = h->nleaf;
    }
    {
        int k = 0;
        auto pf = [&](const void* p, size_t bytes) {
            if (p && bytes >= 16 && k < TreeArgs::MAX_PREFETCH) {
                ta.pf[k] = p;
                ta.pf_bytes[k++] = bytes;
            }
        };
        const OpTables* t = h->tab;
        pf(h->d_m2m_t, sizeof(float) * t->m2m_t.size());
        pf(h->d_l2l_t, sizeof(float) * t->l2l_t.size());
        pf(h->d_entries, h->tasks_bytes);
    }
    d.tree_blocks = tree_blocks(n);
    const int nd = 1 << D;
    d.tree_smem = sizeof(float) * (((3 * (nd + 1) + 1) & ~1) + 6 * nd);
    d.scatter = ScatterArgs{h->d_code, n, h->d_off, h->d_inv, h->d_tmp};
    d.scatter_blocks = (n + 255) / 256;
    d.leaf = LeafSortArgs{h->d_off, h->nleaf, h->d_tmp, h->d_uq, h->d_order, h->d_atoms, h->d_inv, h->d_counts,
                          h->d_leaf_edge};
    d.leaf_blocks = (int)(((long)h->nleaf * 32 + 255) / 256);
    d.fused = D >= 2 && p2m_m2m_smem_bytes(h->P) > 0 && h->nleaf % 8 == 0;
    if (d.fused) {
        d.p2m = P2MArgs{h->d_off, h->nleaf, h->d_atoms, h->Mlev[D], h->Mlev[D - 1], h->d_m2m_t, h->Rpad};
        d.p2m_blocks = h->nleaf / 8;
    } else {
        d.p2m = P2MArgs{h->d_off, h->nleaf, h->d_atoms, h->Mlev[D], nullptr, nullptr, h->Rpad};
        d.p2m_blocks = (h->nleaf + p2m_warps(h->P) - 1) / p2m_warps(h->P);
    }
    const int top_from = D == 1 || h->R > TOP_STAGE_MAX_R ? 1 : std::min(3, d.fused ? D - 1 : D);
    for (int k = d.fused ? D - 2 : D - 1; k >= top_from; k--)
        d.m2m.push_back(M2MArgs{h->Mlev[k + 1], h->Mlev[k], h->d_m2m_t, (int)h->ncell[k], h->R, h->Rpad});
    RootArgs& ra = d.root;
    ra.R = h->R;
    ra.Rpad = h->Rpad;
    ra.m2m = h->d_root_m2m;
    ra.l2l = h->d_root_l2l;
    ra.lattice = h->d_lattice;
    ra.M1 = h->Mlev[1];
    ra.M0 = h->d_M0;
    ra.L0 = h->d_L0;
    ra.M0f = h->Mlev[0];
    ra.L1 = h->Llev[1];
    ra.sc = h->d_sc;
    ra.images = h->prm.images;
    ra.n1 = (int)h->ncell[1];
    TopArgs& top = d.top;
    top.root = ra;
    top.from = top_from;
    top.lattice = h->R <= TOP_LATTICE_MAX_R ? 1 : 0;
    top.Min = h->Mlev[top_from];
    top.M2 = D >= 2 ? h->Mlev[2] : nullptr;
    top.M1 = h->Mlev[1];
    top.m2m_t = h->d_m2m_t;
    top.part = h->d_root_part;
    top.tree_part = h->d_partials;
    top.tree_nblocks = tree_blocks(h->n);
    top.sums = h->d_sums;
    top.fconst = h->d_fconst;
    top.inv_natoms = 1.0 / std::max(h->n, 1);
    top.done = sync + 3;
    top.err = h->d_flags + 2;
    top.umask = (h->shift[0] == 0 ? 4 : 0) | (h->shift[1] == 0 ? 2 : 0) | (h->shift[2] == 0 ? 1 : 0);
    d.top_smem = top_smem_bytes(h->R);
    d.top_staged = h->R <= TOP_STAGE_MAX_R;
    if (h->tc) {
        d.grids = tc_grid_args(h);
        d.grids.root_l2l = h->d_root_l2l;
        d.grids.L0 = h->d_L0;
        d.grids.L1 = h->Llev[1];
        d.grids.root_R = h->R;
        d.grids.root_n1 = (int)h->ncell[1];
        d.grids_blocks = (int)tc_grids_blocks(d.grids);
        TcArgs& t = *h->tca;
        t.tasks = h->d_tc_tasks_v[h->tc_split_v];
        t.atomic = h->tc_split_v > 0 ? 1 : 0;
        t.nstage = h->tc_nstage;
        d.m2l_blocks = h->tc_ntask_v[h->tc_split_v];
        d.m2l_smem = tc_smem_bytes(t);
    }
    if (D >= 2) {
        DownArgs& da = d.down;
        da.nparent = (int)h->ncell[D - 1];
        da.off = h->d_off;
        da.atoms = h->d_atoms;
        for (int k = 0; k <= D; k++) da.L[k] = h->Llev[k];
        da.l2l_t = h->d_l2l_t;
        da.field = h->d_far;
        da.depth = D;
        da.Rpad = h->Rpad;
        da.err = h->d_flags + 2;
        da.wait_limit = WAIT_POLLS_DEFAULT;
    } else {
        d.l2p = L2PArgs{h->d_off, h->nleaf, h->d_atoms, h->Llev[D], h->Rpad, h->d_far};
    }
    FinalArgs& fa = d.fin;
    fa.sc = h->d_sc;
    fa.n = n;
    fa.atoms = h->d_atoms;
    fa.inv = h->d_inv;
    fa.near = h->d_near;
    fa.far = h->d_far;
    fa.fconst = h->d_fconst;
    fa.flags = h->d_flags;
    fa.partials = h->d_partials;
    fa.done = sync + 1;
    fa.zero_after = sync + 2;
    d.fin_blocks = final_blocks(n);
}

// Argument tables of the grouped launches, laid out in one host buffer and
// uploaded in one copy: per group, the systems' argument structs (64-byte
// aligned, for the tensor maps) and the prefix sums of their grid sizes.
struct GroupTable {
    std::vector<uint8_t> host;
    struct Group {
        BatchKernel kind;
        int P = 0;
        size_t args_off = 0, first_off = 0;
        int nsys = 0, nblocks = 0;
        size_t smem = 0;
    };
    std::vector<Group> groups;
    template <typename T>
    void add(BatchKernel kind, int P, size_t smem, const std::vector<const T*>& args, const std::vector<int>& blocks)
    {
        if (args.empty()) return;
        Group g;
        g.kind = kind;
        g.P = P;
        g.smem = smem;
        g.nsys = (int)args.size();
        size_t o = (host.size() + 63) & ~(size_t)63;
        g.args_off = o;
        host.resize(o + sizeof(T) * args.size());
        for (size_t i = 0; i < args.size(); i++) std::memcpy(&host[o + i * sizeof(T)], args[i], sizeof(T));
        o = (host.size() + 15) & ~(size_t)15;
        g.first_off = o;
        host.resize(o + sizeof(int) * (args.size() + 1));
        int acc = 0;
        for (size_t i = 0; i <= args.size(); i++) {
            std::memcpy(&host[o + i * sizeof(int)], &acc, sizeof(int));
            if (i < args.size()) acc += blocks[i];
        }
        g.nblocks = acc;
        if (acc > 0) groups.push_back(g);
    }
};

// The batch step in one captured graph: each kind of kernel runs for every
// system of a far-field lane in one launch (one per order where the kernel is
// templated on the order, or per shared-memory size), the near fields of all
// systems in one persistent kernel beside the far fields.
static int batch_capture(gbfmm_batch* b)
{
    const int ns = b->n_sys;
    std::vector<StepDesc> d(ns);
    for (int i = 0; i < ns; i++) describe_step(b->hs[i], d[i]);
    // Far-field lanes: the orders, heaviest first (atoms x rows^2), each to the
    // least loaded lane; a lane's systems share its grouped launches.
    const int L = std::max(1, std::min(b->far_lanes, (int)b->workers.size()));
    std::vector<int> lane(ns, 0);
    if (L > 1) {
        std::vector<std::pair<double, int>> work;  // (work, order)
        for (int P = 2; P <= MAX_ORDER; P++) {
            double w = 0;
            for (auto& x : d)
                if (x.h->P == P) w += (double)x.h->n * x.h->R * x.h->R;
            if (w > 0) work.push_back({w, P});
        }
        std::sort(work.begin(), work.end(), [](auto& x, auto& y) { return x.first > y.first; });
        std::vector<double> load(L, 0.0);
        int lane_of_P[MAX_ORDER + 1] = {};
        for (auto& wp : work) {
            const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            load[l] += wp.first;
            lane_of_P[wp.second] = l;
        }
        for (int i = 0; i < ns; i++) lane[i] = lane_of_P[d[i].h->P];
    }
    // tables: tree keys; scatter and leaf sort; per lane the upward pass to the
    // tensor-core grids, the tensor-core M2L and the downward pass; the finalize
    // (after the near fields join)
    GroupTable tree, sort, fin;
    std::vector<GroupTable> up(L), m2l(L), down(L);
    {
        std::vector<const TreeArgs*> ta;
        std::vector<const ScatterArgs*> sa;
        std::vector<const LeafSortArgs*> la;
        std::vector<int> tb, sb, lb;
        size_t tsm = 0;
        for (auto& x : d) {
            if (x.h->n <= 0) continue;
            ta.push_back(&x.tree);
            tb.push_back(x.tree_blocks);
            tsm = std::max(tsm, x.tree_smem);
            sa.push_back(&x.scatter);
            sb.push_back(x.scatter_blocks);
        }
        for (auto& x : d) {
            la.push_back(&x.leaf);
            lb.push_back(x.leaf_blocks);
        }
        tree.add(BatchKernel::TREE_KEYS, 0, tsm, ta, tb);
        sort.add(BatchKernel::SCATTER, 0, 0, sa, sb);
        sort.add(BatchKernel::LEAF_SORT, 0, 0, la, lb);
    }
    for (int l = 0; l < L; l++) {
        auto in = [&](const StepDesc& x) { return lane[&x - d.data()] == l; };
        for (int P = 2; P <= MAX_ORDER; P++) {
            std::vector<const P2MArgs*> fa, ua;
            std::vector<int> fb, ub;
            for (auto& x : d)
                if (in(x) && x.h->P == P) {
                    (x.fused ? fa : ua).push_back(&x.p2m);
                    (x.fused ? fb : ub).push_back(x.p2m_blocks);
                }
            up[l].add(BatchKernel::P2M_M2M, P, p2m_m2m_smem_bytes(P), fa, fb);
            up[l].add(BatchKernel::P2M, P, p2m_smem_bytes(P), ua, ub);
        }
        size_t rounds = 0;
        for (auto& x : d)
            if (in(x)) rounds = std::max(rounds, x.m2m.size());
        for (size_t r = 0; r < rounds; r++) {
            std::vector<const M2MArgs*> ma;
            std::vector<int> mb;
            size_t sm = 0;
            for (auto& x : d)
                if (in(x) && r < x.m2m.size()) {
                    ma.push_back(&x.m2m[r]);
                    mb.push_back(x.m2m[r].nparent * ((x.m2m[r].R + 31) / 32));
                    sm = std::max(sm, sizeof(float) * 8 * (size_t)x.m2m[r].R);
                }
            up[l].add(BatchKernel::M2M, 0, sm, ma, mb);
        }
        std::vector<int> Rs;
        for (auto& x : d)
            if (in(x)) Rs.push_back(x.h->R);
        std::sort(Rs.begin(), Rs.end());
        Rs.erase(std::unique(Rs.begin(), Rs.end()), Rs.end());
        for (int R : Rs) {
            std::vector<const TopArgs*> ta;
            std::vector<int> tb;
            bool staged = false;
            size_t sm = 0;
            for (auto& x : d)
                if (in(x) && x.h->R == R) {
                    ta.push_back(&x.top);
                    tb.push_back((int)x.h->ncell[1]);
                    staged = x.top_staged;
                    sm = x.top_smem;
                }
            up[l].add(staged ? BatchKernel::TOP_STAGED : BatchKernel::TOP_UNSTAGED, 0, sm, ta, tb);
        }
        std::vector<const RootArgs*> ra;
        std::vector<int> rb;
        for (auto& x : d)
            if (in(x) && !x.top.lattice) {
                ra.push_back(&x.root);
                rb.push_back((x.h->R + 7) / 8);
            }
        up[l].add(BatchKernel::ROOT_LATTICE, 0, 0, ra, rb);
        std::vector<const TcGridArgs*> ga;
        std::vector<int> gb;
        for (auto& x : d)
            if (in(x) && x.h->tc) {
                ga.push_back(&x.grids);
                gb.push_back(x.grids_blocks);
            }
        up[l].add(BatchKernel::TC_GRIDS, 0, 0, ga, gb);
        std::vector<size_t> sms;
        for (auto& x : d)
            if (in(x) && x.h->tc) sms.push_back(x.m2l_smem);
        std::sort(sms.begin(), sms.end());
        sms.erase(std::unique(sms.begin(), sms.end()), sms.end());
        for (size_t sm : sms) {
            std::vector<const TcArgs*> ma;
            std::vector<int> mb;
            for (auto& x : d)
                if (in(x) && x.h->tc && x.m2l_smem == sm) {
                    ma.push_back(x.h->tca);
                    mb.push_back(x.m2l_blocks);
                }
            m2l[l].add(BatchKernel::M2L_TC, 0, sm, ma, mb);
        }
        for (int P = 2; P <= MAX_ORDER; P++) {
            std::vector<const DownArgs*> da;
            std::vector<const L2PArgs*> la;
            std::vector<int> db, lb;
            for (auto& x : d)
                if (in(x) && x.h->P == P) {
                    if (x.h->D >= 2) {
                        da.push_back(&x.down);
                        db.push_back(x.down.nparent);
                    } else {
                        la.push_back(&x.l2p);
                        lb.push_back((x.h->nleaf + 3) / 4);
                    }
                }
            down[l].add(BatchKernel::DOWN, P, down_smem_bytes(P), da, db);
            down[l].add(BatchKernel::L2P, P, 0, la, lb);
        }
    }
    {
        std::vector<const FinalArgs*> fa;
        std::vector<int> fb;
        for (auto& x : d)
            if (x.h->n > 0) {
                fa.push_back(&x.fin);
                fb.push_back(x.fin_blocks);
            }
        fin.add(BatchKernel::FINALIZE, 0, 0, fa, fb);
    }
    // one device buffer for every table
    std::vector<GroupTable*> tabs = {&tree, &sort, &fin};
    for (int l = 0; l < L; l++) {
        tabs.push_back(&up[l]);
        tabs.push_back(&m2l[l]);
        tabs.push_back(&down[l]);
    }
    std::vector<size_t> base(tabs.size());
    size_t total = 0;
    for (size_t t = 0; t < tabs.size(); t++) {
        base[t] = total;
        total = (total + tabs[t]->host.size() + 255) & ~(size_t)255;
    }
    if (total > b->group_bytes) {
        if (b->group_buf) cudaFree(b->group_buf);
        b->group_buf = nullptr;
        b->group_bytes = 0;
        CK(cudaMalloc(&b->group_buf, std::max<size_t>(total, 256)));
        b->group_bytes = std::max<size_t>(total, 256);
    }
    for (size_t t = 0; t < tabs.size(); t++)
        if (!tabs[t]->host.empty())
            CK(cudaMemcpy((char*)b->group_buf + base[t], tabs[t]->host.data(), tabs[t]->host.size(),
                          cudaMemcpyHostToDevice));
    auto run = [&](const GroupTable& tab, cudaStream_t st) {
        const size_t t = std::find(tabs.begin(), tabs.end(), &tab) - tabs.begin();
        const char* dev = (const char*)b->group_buf + base[t];
        for (const auto& g : tab.groups) {
            const void* args = dev + g.args_off;
            const int* first = reinterpret_cast<const int*>(dev + g.first_off);
            if (g.kind == BatchKernel::TC_GRIDS || g.kind == BatchKernel::M2L_TC)
                launch_batch_tc(g.kind, args, first, g.nsys, g.nblocks, g.smem, st);
            else
                launch_batch(g.kind, g.P, args, first, g.nsys, g.nblocks, g.smem, st);
        }
    };
    const long launches0 = g_kernel_launches.load();
    const bool forked = L > 1 || b->far_prio;
    std::vector<cudaStream_t> ls(L, b->master);
    if (forked)
        for (int l = 0; l < L; l++) ls[l] = b->far_prio ? b->workers_hi[l] : b->workers[l];
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(b->master, cudaStreamCaptureModeThreadLocal));
    CK(cudaEventRecord(b->ein, b->master));
    // 1) every system's tree (one launch per kernel); the leaf scan of systems too
    //    large for the tree kernel's epilogue runs between the keys and the scatter
    run(tree, b->master);
    for (auto& x : d)
        if (x.h->n > 0 && !x.tree.off)
            launch_exclusive_scan(x.h->d_counts, x.h->d_off, x.h->nleaf, x.h->d_scan, b->master);
    run(sort, b->master);
    CK(cudaEventRecord(b->ev_near, b->master));
    // 2) the far fields, lane by lane: one launch per kind (per order or shared-
    //    memory size); systems with the FP32 M2L keep their own contraction and
    //    root L2L
    for (int l = 0; l < L; l++) {
        if (forked) CK(cudaStreamWaitEvent(ls[l], b->ev_near, 0));
        run(up[l], ls[l]);
        CK(cudaEventRecord(b->ev_up[l], ls[l]));
        run(m2l[l], ls[l]);
        for (int i = 0; i < ns; i++)
            if (lane[i] == l && !d[i].h->tc) {
                ContractArgs a = contract_args(d[i].h, OP_M2L, 2, false, d[i].h->m2l_task0);
                launch_contract(a, d[i].h->m2l_ntask, ls[l]);
                launch_root_l2l(d[i].root, ls[l]);
            }
        if (b->near_after == 2) CK(cudaEventRecord(b->ev_up[l], ls[l]));
        run(down[l], ls[l]);
        if (forked) CK(cudaEventRecord(b->ev[l], ls[l]));
    }
    // 3) all near fields: one persistent kernel over every system's leaves, from
    //    the tree on, or from the far fields' M2L on (near_after)
    CK(cudaStreamWaitEvent(b->near_stream, b->ev_near, 0));
    if (b->near_after > 0)
        for (int l = 0; l < L; l++) CK(cudaStreamWaitEvent(b->near_stream, b->ev_up[l], 0));
    CK(cudaMemsetAsync(b->p2p.counter, 0, sizeof(int), b->near_stream));
    launch_p2p_batch(b->p2p, b->p2p_shape, b->p2p_per_sm, b->near_stream);
    cudaEvent_t ev_nf = b->ev_tree[0];
    CK(cudaEventRecord(ev_nf, b->near_stream));
    // 4) join the lanes and the near fields, then every system's forces,
    //    potentials and energy
    if (forked)
        for (int l = 0; l < L; l++) CK(cudaStreamWaitEvent(b->master, b->ev[l], 0));
    CK(cudaStreamWaitEvent(b->master, ev_nf, 0));
    run(fin, b->master);
    for (auto& x : d)
        if (x.h->n <= 0) CK(cudaMemsetAsync(x.h->d_energy, 0, sizeof(double), b->master));
    cudaError_t e = cudaStreamEndCapture(b->master, &g);
    if (e != cudaSuccess) return fail(GBFMM_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->gexec, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(GBFMM_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(e));
    b->step_launches = (int)(g_kernel_launches.load() - launches0);
    return GBFMM_OK;
}

extern "C" int gbfmm_batch_step_launches(gbfmm_batch* b, int* n)
{
    if (!b || !n) return fail(GBFMM_ERR_ARG, "NULL argument");
    *n = b->step_launches;
    return GBFMM_OK;
}

extern "C" int gbfmm_batch_execute_device(gbfmm_batch* b, const void* d_coords, const void* d_charges,
                                          const float* box_edges, void* stream)
{
    if (!b || !box_edges || (b->natoms > 0 && (!d_coords || !d_charges))) return fail(GBFMM_ERR_ARG, "NULL argument");
    if (b->ev_sc) cudaEventSynchronize(b->ev_sc);  // the previous batch's copy of h_sc has been made
    for (int i = 0; i < b->n_sys; i++) {
        gbfmm_handle* h = b->hs[i];
        float box[9] = {box_edges[i], 0, 0, 0, box_edges[i], 0, 0, 0, box_edges[i]};
        int rc = set_box(h, box, (const float*)d_coords + 3 * (size_t)b->off[i]);
        if (rc) return rc;
        b->h_sc[i] = *h->h_sc;
    }
    cudaStream_t us = (cudaStream_t)stream;
    CK(cudaEventRecord(b->ein, us));
    CK(cudaStreamWaitEvent(b->master, b->ein, 0));
    if (d_charges != b->d_q)
        CK(cudaMemcpyAsync(b->d_q, d_charges, sizeof(float) * b->natoms, cudaMemcpyDeviceToDevice, b->master));
    CK(cudaMemcpyAsync(b->d_sc, b->h_sc, sizeof(StepConst) * b->n_sys, cudaMemcpyHostToDevice, b->master));
    CK(cudaEventRecord(b->ev_sc, b->master));
    if (!b->gexec) {
        int rc = batch_capture(b);
        if (rc) return rc;
    }
    CK(cudaGraphLaunch(b->gexec, b->master));
    CK(cudaEventRecord(b->eout, b->master));
    CK(cudaStreamWaitEvent(us, b->eout, 0));
    b->have_result = true;
    return GBFMM_OK;
}

// ---- batch autotuner: the near-field kernel's warp-step shape and CTAs per SM
// and, for the tensor-core systems, a batch-wide M2L entry split and pipeline
// depth, chosen by timing replays of the batch graph on the caller's inputs.

static int apply_batch_tuning(gbfmm_batch* b, int shape, int per_sm, int split_v, int nstage)
{
    if (shape < 0 || shape >= p2p_batch_shapes()) return fail(GBFMM_ERR_ARG, "batch p2p shape %d", shape);
    if (per_sm < 0 || per_sm > 5)
        return fail(GBFMM_ERR_ARG, "batch p2p residency %d outside [0,5] (0: a CTA per leaf)", per_sm);
    if (split_v >= TC_NSPLIT) return fail(GBFMM_ERR_ARG, "m2l split");
    for (gbfmm_handle* h : b->hs)
        if (h->tc && split_v >= 0 && h->tc_ntask_v[split_v] == 0)
            return fail(GBFMM_ERR_ARG, "m2l split %d unavailable (deterministic batch)", 1 << split_v);
    if (nstage < 0) return fail(GBFMM_ERR_ARG, "m2l stages %d", nstage);
    if (b->gexec) CK(cudaStreamSynchronize(b->master));
    b->p2p_shape = shape;
    b->p2p_per_sm = per_sm;
    b->m2l_split_v = split_v;
    b->m2l_stages = nstage;
    for (gbfmm_handle* h : b->hs) {
        if (!h->tc) continue;
        if (split_v >= 0) h->tc_split_v = split_v;
        if (nstage > 0) {
            const TcPlan& pl = h->tab->tc;
            h->tc_nstage = std::max(1, std::min(nstage, tc_max_stages(pl.k_atoms, pl.img_bytes, h->tca->nprod) /
                                                             h->tca->group));
        }
    }
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    return GBFMM_OK;
}

extern "C" int gbfmm_batch_set_tuning(gbfmm_batch* b, int p2p_shape, int p2p_per_sm, int m2l_split, int m2l_stages)
{
    if (!b) return fail(GBFMM_ERR_ARG, "batch is NULL");
    int v = -1;
    if (m2l_split != 0) {
        v = 0;
        while (v < TC_NSPLIT - 1 && (1 << v) < m2l_split) v++;
        if (m2l_split < 1 || (1 << v) != m2l_split) return fail(GBFMM_ERR_ARG, "m2l split %d is not 0, 1, 2, 4 or 8", m2l_split);
    }
    return apply_batch_tuning(b, p2p_shape, p2p_per_sm, v, m2l_stages);
}

extern "C" int gbfmm_batch_get_tuning(gbfmm_batch* b, int* p2p_shape, int* p2p_per_sm, int* m2l_split, int* m2l_stages)
{
    if (!b) return fail(GBFMM_ERR_ARG, "batch is NULL");
    if (p2p_shape) *p2p_shape = b->p2p_shape;
    if (p2p_per_sm) *p2p_per_sm = b->p2p_per_sm;
    if (m2l_split) *m2l_split = b->m2l_split_v >= 0 ? 1 << b->m2l_split_v : 0;
    if (m2l_stages) *m2l_stages = b->m2l_stages;
    return GBFMM_OK;
}

static int apply_batch_schedule(gbfmm_batch* b, int far_lanes, int far_prio, int near_after)
{
    if (far_lanes < 1 || far_lanes > (int)b->workers.size())
        return fail(GBFMM_ERR_ARG, "far lanes %d outside [1,%d]", far_lanes, (int)b->workers.size());
    if (near_after < 0 || near_after > 2) return fail(GBFMM_ERR_ARG, "near_after %d outside [0,2]", near_after);
    if (b->gexec) {
        CK(cudaStreamSynchronize(b->master));
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    b->far_lanes = far_lanes;
    b->far_prio = far_prio != 0;
    b->near_after = near_after;
    return GBFMM_OK;
}

extern "C" int gbfmm_batch_set_schedule(gbfmm_batch* b, int far_lanes, int far_prio, int near_after)
{
    if (!b) return fail(GBFMM_ERR_ARG, "batch is NULL");
    return apply_batch_schedule(b, far_lanes, far_prio, near_after);
}

extern "C" int gbfmm_batch_get_schedule(gbfmm_batch* b, int* far_lanes, int* far_prio, int* near_after)
{
    if (!b) return fail(GBFMM_ERR_ARG, "batch is NULL");
    if (far_lanes) *far_lanes = b->far_lanes;
    if (far_prio) *far_prio = b->far_prio ? 1 : 0;
    if (near_after) *near_after = b->near_after;
    return GBFMM_OK;
}

extern "C" int gbfmm_batch_autotune(gbfmm_batch* b, const void* d_coords, const void* d_charges,
                                    const float* box_edges, int reps, float* best_ms)
{
    if (!b || !box_edges || (b->natoms > 0 && (!d_coords || !d_charges))) return fail(GBFMM_ERR_ARG, "NULL argument");
    if (reps <= 0) reps = 3;
    L2Flush flush;  // each timed step starts from a flushed L2
    std::vector<cudaEvent_t> e0(reps), e1(reps);
    for (int i = 0; i < reps; i++) {
        CK(cudaEventCreate(&e0[i]));
        CK(cudaEventCreate(&e1[i]));
    }
    int err = GBFMM_OK;
    auto measure = [&](int sh, int ps, int sv, int ns) -> float {
        if (apply_batch_tuning(b, sh, ps, sv, ns) != GBFMM_OK) return 1e30f;
        for (int i = 0; i < 2 && err == GBFMM_OK; i++)
            err = gbfmm_batch_execute_device(b, d_coords, d_charges, box_edges, b->master);
        if (err) return 1e30f;
        for (int i = 0; i < reps && err == GBFMM_OK; i++) {
            flush.run(b->master);
            cudaEventRecord(e0[i], b->master);
            err = gbfmm_batch_execute_device(b, d_coords, d_charges, box_edges, b->master);
            cudaEventRecord(e1[i], b->master);
        }
        if (cudaEventSynchronize(e1[reps - 1]) != cudaSuccess) err = GBFMM_ERR_CUDA;
        float tot = 0.f;
        for (int i = 0; i < reps && !err; i++) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0[i], e1[i]);
            tot += ms;
        }
        return err ? 1e30f : tot / reps;
    };
    int bs = b->p2p_shape, bp = b->p2p_per_sm, bv = b->m2l_split_v, bn = b->m2l_stages;
    float bt = measure(bs, bp, bv, bn);
    // coordinate search: near-field shape and CTAs per SM, then M2L split, then M2L depth
    for (int sh = 0; sh < p2p_batch_shapes() && !err; sh++)
        for (int ps = 0; ps <= 5 && !err; ps++) {
            if (ps == 1 || (sh == bs && ps == bp)) continue;
            const float t = measure(sh, ps, bv, bn);
            if (t < bt) { bt = t; bs = sh; bp = ps; }
        }
    bool any_tc = false;
    for (gbfmm_handle* h : b->hs) any_tc |= h->tc;
    if (any_tc) {
        for (int sv = 0; sv < TC_NSPLIT && !err; sv++) {
            bool ok = sv != bv;
            for (gbfmm_handle* h : b->hs) ok &= !h->tc || h->tc_ntask_v[sv] > 0;
            if (!ok) continue;
            const float t = measure(bs, bp, sv, bn);
            if (t < bt) { bt = t; bv = sv; }
        }
        for (int ns = 1; ns <= 4 && !err; ns++) {
            if (ns == bn) continue;
            const float t = measure(bs, bp, bv, ns);
            if (t < bt) { bt = t; bn = ns; }
        }
    }
    // schedule: far-field lanes (up to one per expansion order), their stream
    // priority, and when the near-field kernel starts
    {
        bool seen[MAX_ORDER + 1] = {};
        int norders = 0;
        for (gbfmm_handle* h : b->hs)
            if (!seen[h->P]) {
                seen[h->P] = true;
                norders++;
            }
        const int maxl = std::max(1, std::min(norders, (int)b->workers.size()));
        int bl = b->far_lanes, bq = b->far_prio ? 1 : 0, ba = b->near_after;
        if (!err && apply_batch_tuning(b, bs, bp, bv, bn) == GBFMM_OK) {
            auto measure_sched = [&](int l, int q, int a) -> float {
                if (apply_batch_schedule(b, l, q, a) != GBFMM_OK) return 1e30f;
                return measure(bs, bp, bv, bn);
            };
            bt = measure_sched(bl, bq, ba);
            for (int l = 1; l <= maxl && !err; l++)
                for (int q = 0; q <= 1 && !err; q++)
                    for (int a = 0; a <= 1 && !err; a++) {
                        if (l == bl && q == bq && a == ba) continue;
                        const float t = measure_sched(l, q, a);
                        if (t < bt) { bt = t; bl = l; bq = q; ba = a; }
                    }
        }
        if (!err) err = apply_batch_schedule(b, bl, bq, ba);
        // the near field's residency again, under the chosen schedule
        for (int ps = 0; ps <= 5 && !err; ps++) {
            if (ps == 1 || ps == bp) continue;
            const float t = measure(bs, ps, bv, bn);
            if (t < bt) { bt = t; bp = ps; }
        }
    }
    for (int i = 0; i < reps; i++) {
        cudaEventDestroy(e0[i]);
        cudaEventDestroy(e1[i]);
    }
    if (err) return err;
    const int rc = apply_batch_tuning(b, bs, bp, bv, bn);
    if (rc) return rc;
    if (best_ms) *best_ms = bt;
    return GBFMM_OK;
}

static int batch_check(gbfmm_batch* b);

extern "C" int gbfmm_batch_execute(gbfmm_batch* b, const float* coords, const float* charges, const float* box_edges,
                                   float* forces, float* potentials, double* energies)
{
    if (!b || !box_edges || (b->natoms > 0 && (!coords || !charges))) return fail(GBFMM_ERR_ARG, "NULL argument");
    for (int i = 0; i < b->n_sys; i++)
        for (int k = b->off[i]; k < b->off[i + 1]; k++)
            if (!std::isfinite(charges[k])) return fail(GBFMM_ERR_COORD, "charge %d is not finite", k);
    CK(cudaMemcpyAsync(b->d_coords, coords, sizeof(float) * 3 * b->natoms, cudaMemcpyHostToDevice, b->master));
    CK(cudaMemcpyAsync(b->d_q, charges, sizeof(float) * b->natoms, cudaMemcpyHostToDevice, b->master));
    int rc = gbfmm_batch_execute_device(b, b->d_coords, b->d_q, box_edges, b->master);
    if (rc) return rc;
    if (forces) CK(cudaMemcpyAsync(forces, b->d_forces, sizeof(float) * 3 * b->natoms, cudaMemcpyDeviceToHost, b->master));
    if (potentials) CK(cudaMemcpyAsync(potentials, b->d_pots, sizeof(float) * b->natoms, cudaMemcpyDeviceToHost, b->master));
    if (energies) CK(cudaMemcpyAsync(energies, b->d_energy, sizeof(double) * b->n_sys, cudaMemcpyDeviceToHost, b->master));
    CK(cudaStreamSynchronize(b->master));
    return batch_check(b);
}

// Reads every system's step flags (word 0 non-finite input, words 1-3 a bounded
// wait of the tensor-core M2L, the upper-tree or the near-field kernel gave up); on an error
// clears the flags and the step counters, as fetch() does for one system.
static int batch_check(gbfmm_batch* b)
{
    CK(cudaStreamSynchronize(b->master));
    int rc = GBFMM_OK;
    for (gbfmm_handle* h : b->hs) {
        int fl[4];
        CK(cudaMemcpy(fl, h->d_flags, sizeof(fl), cudaMemcpyDeviceToHost));
        if (fl[0] || fl[1] || fl[2] || fl[3]) {
            CK(cudaMemset(h->d_flags, 0, sizeof(int) * 4));
            if (fl[1] || fl[2] || fl[3]) CK(cudaMemset(h->d_counts, 0, sizeof(int) * (h->nleaf + 1 + 4)));
            if (rc == GBFMM_OK)
                rc = fail(fl[1] || fl[2] || fl[3] ? GBFMM_ERR_TIMEOUT : GBFMM_ERR_COORD,
                          fl[1]   ? "a bounded device wait in a system's tensor-core M2L gave up"
                          : fl[2] ? "a bounded device wait in a system's upper-tree or downward-pass kernel gave up"
                          : fl[3] ? "a bounded device wait in a system's near-field kernel gave up"
                                  : "a system of the batch has a non-finite coordinate");
        }
    }
    if (rc != GBFMM_OK) b->have_result = false;
    return rc;
}

extern "C" int gbfmm_batch_status(gbfmm_batch* b)
{
    if (!b) return fail(GBFMM_ERR_ARG, "batch is NULL");
    return batch_check(b);
}

extern "C" int gbfmm_batch_device_outputs(gbfmm_batch* b, void** f, void** p, void** e)
{
    if (!b) return fail(GBFMM_ERR_ARG, "batch is NULL");
    if (f) *f = b->d_forces;
    if (p) *p = b->d_pots;
    if (e) *e = b->d_energy;
    return GBFMM_OK;
}

extern "C" int gbfmm_batch_destroy(gbfmm_batch* b)
{
    if (!b) return fail(GBFMM_ERR_ARG, "batch is NULL");
    if (b->master) cudaStreamSynchronize(b->master);
    free_batch(b);
    return GBFMM_OK;
}
