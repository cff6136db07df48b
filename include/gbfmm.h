/*
 * gbfmm.h -- C ABI of the GB300-native FMM Coulomb solver.
 *
 * Drop-in for the solver that mdrun reaches through the fork's Coulomb-solver
 * plugin interface, coulomb_solver::BaseSolver
 * (src/gromacs/coulomb_solvers/basesolver.h:43-90), as implemented for the GPU
 * FMM by zeta_fmm::ZetaFmmSolver (src/gromacs/zeta_fmm/zeta_fmm_solver.cpp).
 * Plain C types only: host pointers, device pointers as void*, a CUDA stream as
 * void*.  Every call returns a gbfmm_status; nothing calls exit().
 *
 * Units follow GROMACS: nm, e, kJ/mol; forces kJ/mol/nm.
 */
#ifndef GBFMM_H
#define GBFMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference has none: CUDA errors print and exit(-1)
 * (src/gromacs/zeta_fmm/type.h:23-28), an unknown solver exits(0)
 * (src/gromacs/coulomb_solvers/executer.h:55-59). */
typedef enum gbfmm_status {
    GBFMM_OK = 0,
    GBFMM_ERR_ARG = 1,        /* invalid argument (null pointer, size, order, depth) */
    GBFMM_ERR_BOX = 2,        /* box not cubic, not positive or not finite */
    GBFMM_ERR_COORD = 3,      /* NaN/Inf coordinate or charge */
    GBFMM_ERR_CUDA = 4,       /* CUDA runtime error (message via gbfmm_last_error) */
    GBFMM_ERR_NOMEM = 5,      /* device or host allocation failed, or the arena cap was hit */
    GBFMM_ERR_UNSUPPORTED = 6,/* feature not built (e.g. rega > 0, tensor M2L for this order) */
    GBFMM_ERR_STATE = 7,      /* call out of order (e.g. forces before execute) */
    GBFMM_ERR_TIMEOUT = 8,    /* a bounded device wait gave up; the context stays usable */
    GBFMM_ERR_NOT_NEUTRAL = 9 /* reserved */
} gbfmm_status;

/* M2L arithmetic. */
typedef enum gbfmm_precision {
    GBFMM_PREC_FP32 = 0,      /* plain FP32 CUDA-core M2L */
    GBFMM_PREC_BF16X3 = 1,    /* tcgen05 tensor-core M2L, split bf16 hi+lo (3 products), FP32 accumulate */
    GBFMM_PREC_BF16X1 = 2     /* tcgen05 tensor-core M2L, single bf16 product, FP32 accumulate */
} gbfmm_precision;

/* Solver parameters.  Defaults (gbfmm_params_default) are the reference's
 * constants: P=10, max_depth=3, images=4, rega=0 (zeta_fmm_solver.cpp:10-13)
 * and MAC scale 0.4 (gpu_solver.cu:46). */
typedef struct gbfmm_params {
    int order;          /* expansion order P, 2..16 */
    int max_depth;      /* uniform tree depth, 1..7 */
    int images;         /* periodic lattice levels: 0 = free space, 1 = 27 near shifts only, >=2 adds far images */
    double theta;       /* MAC scale; only 0.4 is supported (stencils are precomputed for it) */
    double rega;        /* regularisation width; only 0 is supported */
    int precision;      /* gbfmm_precision */
    int m2l_tile;       /* 0 = autotuned, else targets per M2L tile (32 or 64) */
    int m2l_split;      /* 0 = autotuned, else entry splits per M2L tile (1..16) */
    int flags;          /* GBFMM_FLAG_* */
    int aspect_z;       /* box shape: 1 (or 0) = cube; 2 = slab with Lx = Ly and Lz = 2 Lx.  A slab is
                           solved as the periodic cube of edge Lz that holds it twice along x and y (the
                           same periodic charge density): the tree's root is that cube (max_depth counts
                           from it, leaves of edge Lz / 2^max_depth), and only the box's own cells are
                           stored and computed.  The reference takes box[XX][XX] as the period of a cube
                           (zeta_fmm_solver.cpp:38-40) and has no slab. */
} gbfmm_params;

#define GBFMM_FLAG_NO_GRAPH 1        /* launch the step kernel by kernel instead of replaying a CUDA graph */
#define GBFMM_FLAG_DETERMINISTIC 2   /* no floating-point atomics in M2L (m2l_split forced to 1) */
#define GBFMM_FLAG_HOST_COPY 4       /* gbfmm_execute copies through device buffers even where the device
                                        reads pageable host memory (default there: in place, no copies) */

typedef struct gbfmm_handle gbfmm_handle;

void gbfmm_params_default(gbfmm_params* p);
const char* gbfmm_status_string(int status);
/* Last error message of the calling thread (static storage; valid until the next call). */
const char* gbfmm_last_error(void);
const char* gbfmm_version(void);

/* Constructor: replaces ZetaFmmSolver::ZetaFmmSolver + BaseSolver::BaseSolver
 * (zeta_fmm_solver.cpp:6-14, basesolver.h:46-52).  natoms = t_mdatoms::homenr. */
int gbfmm_create(const gbfmm_params* params, int natoms, gbfmm_handle** out);
int gbfmm_destroy(gbfmm_handle* h);

/* BaseSolver::set_parameter (basesolver.h:56-61): atom count and chargeA.
 * Charges are copied (the reference borrows them and reads them in execute). */
int gbfmm_set_charges(gbfmm_handle* h, int natoms, const float* charges);

/* BaseSolver::execute (basesolver.h:67; zeta_fmm_solver.cpp:16-64): host
 * coordinates (float[3*natoms], nm) and the box (float[9], row-major 3x3, nm;
 * rectangular, of the handle's shape: cubic, or Lx = Ly and Lz = 2 Lx for
 * aspect_z = 2; the reference uses box[XX][XX] as the period of a cube).  Synchronous,
 * like the reference: results are on the host when it returns.  On a device
 * that reads pageable host memory coherently (GB300 over NVLink-C2C) the step
 * reads 'coords' in place and writes the results straight into the handle's
 * pinned host buffers, with no staging copies (GBFMM_FLAG_HOST_COPY turns this
 * off); elsewhere the coordinates and results are copied. */
int gbfmm_execute(gbfmm_handle* h, const float* coords, const float* box, int verbose);

/* Device-resident execute: d_coords float[3*natoms] on the device, results left
 * on the device (see gbfmm_device_outputs).  Asynchronous on 'stream'
 * (cudaStream_t, NULL = default stream). */
int gbfmm_execute_device(gbfmm_handle* h, const void* d_coords, const float* box, void* stream);

/* Device pointers of the results of the last gbfmm_execute_device (and of a
 * gbfmm_execute that copied), in input atom order: forces float[3*natoms]
 * (kJ/mol/nm), potentials float[natoms] (kJ/mol/e), energy double[1] (kJ/mol). */
int gbfmm_device_outputs(gbfmm_handle* h, void** d_forces, void** d_potentials, void** d_energy);

/* BaseSolver::add_force (basesolver.h:72; zeta_fmm_solver.cpp:66-76): adds the
 * Coulomb forces to a host float[3*natoms] array. */
int gbfmm_add_forces(gbfmm_handle* h, float* forces);
int gbfmm_get_forces(gbfmm_handle* h, float* forces);
int gbfmm_get_potentials(gbfmm_handle* h, float* potentials);

/* BaseSolver::get_energy (basesolver.h:77).  The reference returns zeros
 * (zeta_fmm_solver.cpp:109-115); this returns 0.5*sum(q*phi) as the legacy
 * zeta_fmm::FMM::get_energy does (src/gromacs/zeta_fmm/fmm.cpp:89-98). */
int gbfmm_get_energy(gbfmm_handle* h, double* coulomb_energy);

/* Coulomb virial of the last execute, Xi = -1/2 sum over pairs (periodic images
 * included) of r_ij (x) F_ij, kJ/mol, row-major 3 x 3, tin-foil boundary: what
 * mdrun's ForceWithVirial takes for a force provider with its own virial
 * (src/gromacs/mdlib/sim_util.cpp:2085), where the reference's plugin adds forces
 * only (zeta_fmm_solver.cpp:66-76).  Computed on request by an extra pass over
 * the step's tree, expansions and fields: -1/2 sum_i r_i (x) F_i, the forces of
 * the interactions that cross the box (near-field and M2L stencil entries that
 * wrap, the far lattice) weighted by their image shift, and the tin-foil term.
 * The first call on a handle allocates its buffers. */
int gbfmm_get_virial(gbfmm_handle* h, double* virial);

/* BaseSolver::compare_forces (basesolver.h:82; zeta_fmm_solver.cpp:78-107):
 * relative L2 force error sqrt(sum|f-g|^2 / sum|g|^2) against host forces g.
 * Returns GBFMM_ERR_COORD (and l2f = NaN) if a result is NaN, where the
 * reference prints "have nan!". */
int gbfmm_compare_forces(gbfmm_handle* h, const float* ref_forces, double* l2f);

/* Per-stage device times of the last execute (ms, CUDA events), when built with
 * timing enabled by gbfmm_set_timing(h, 1); the stages then run one after
 * another (no near/far overlap).  Stages: tree; p2m (with the M2M of the leaf
 * parents where fused); m2m (the remaining per-level M2M launches); root (upper
 * tree, FP64 root and lattice); m2l (bf16 source grids and root L2L, M2L); l2l
 * (the fused downward pass of L2L and L2P at depth >= 2); l2p (depth 1 only);
 * p2p; finalize. */
int gbfmm_set_timing(gbfmm_handle* h, int enable);
int gbfmm_stage_times(gbfmm_handle* h, float* ms, int n_max, int* n_out);
const char* gbfmm_stage_name(int stage);
/* Number of device kernels one step launches (counted when the step is enqueued). */
int gbfmm_step_launches(gbfmm_handle* h, int* n);

/* ---- tree and interaction lists (integer parity with the reference) ---- */

/* Body order of the last execute: order[i] = input index of the body at sorted
 * position i (CompleteBalancedOctree::build, tree.cpp:13-99), and the body range
 * of every leaf in BFS cell order (leaf_off[k], leaf_num[k] for leaf k). */
int gbfmm_get_tree(gbfmm_handle* h, int* order, int* leaf_off, int* leaf_num);

/* Interaction lists as the reference's Traverser produces them
 * (traverser.cpp:47-214): entries grouped by ascending target cell, in traversal
 * order within a target.  which: 0 = P2P, 1 = M2L.  Cell indices are the
 * reference's BFS indices; image cells follow the tree cells.  offsets are the
 * periodic shift of each source in units of the period (integers).  Two-call
 * protocol: pass NULL arrays to get the count. */
int gbfmm_get_lists(gbfmm_handle* h, int which, long* count, int* target, int* source, int* offset3);
/* The same lists without a handle (host only): tree depth and image levels. */
int gbfmm_lists(int max_depth, int images, int which, long* count, int* target, int* source, int* offset3);

/* ---- learned parameter selection ---- */

/* Per-step statistics of a system (no counterpart in the reference, which fixes
 * P=10 and depth 3, zeta_fmm_solver.cpp:10-11): GBFMM_NFEAT floats -- log N,
 * log density, log L, mean q^2, net-charge and dipole ratios, the body
 * occupancy histograms of octree levels 2..6, and the box shape (log2 Lz/Lx: a
 * cube or a slab) -- computed on the GPU from device coordinates and charges.
 * Written to host memory 'features'. */
#define GBFMM_NFEAT 57
int gbfmm_features(const void* coords, const void* charges, int natoms, const float* box, float* features,
                   void* stream);

/* A small MLP (n_in -> n_hidden -> n_hidden -> n_out, tanh) whose forward,
 * backward and Adam kernels are this library's own.  Parameters are laid out as
 * W1 b1 W2 b2 W3 b3 (row-major W[out][in]). */
typedef struct gbfmm_mlp gbfmm_mlp;
int gbfmm_mlp_create(int n_in, int n_hidden, int n_out, unsigned long long seed, gbfmm_mlp** out);
int gbfmm_mlp_destroy(gbfmm_mlp* m);
int gbfmm_mlp_num_params(gbfmm_mlp* m, int* n);
int gbfmm_mlp_get_params(gbfmm_mlp* m, float* params);
int gbfmm_mlp_set_params(gbfmm_mlp* m, const float* params);
int gbfmm_mlp_set_normalization(gbfmm_mlp* m, const float* x_mean, const float* x_std, const float* y_mean,
                                const float* y_std);
/* Raw network on host rows x[B][n_in] -> y[B][n_out]. */
int gbfmm_mlp_forward(gbfmm_mlp* m, const float* x, int batch, float* y);
/* Raw network: loss = mean_b sum_j (y - t)^2 and its gradient (grad may be NULL). */
int gbfmm_mlp_loss_grad(gbfmm_mlp* m, const float* x, const float* t, int batch, double* loss, float* grad);
/* Adam training on normalised data (the stored normalisation is applied). */
int gbfmm_mlp_train(gbfmm_mlp* m, const float* x, const float* t, int n, int epochs, int batch, float lr,
                    unsigned long long seed, double* final_loss);
/* Prediction in physical units (normalisation applied to inputs and outputs). */
int gbfmm_mlp_predict(gbfmm_mlp* m, const float* x, int batch, float* y);
/* Versioned weights file with an FNV-1a checksum; load rejects corrupted files. */
int gbfmm_mlp_save(gbfmm_mlp* m, const char* path);
int gbfmm_mlp_load(const char* path, gbfmm_mlp** out);
/* Input row of the tuner network: statistics ++ encoding of (order, depth, precision). */
int gbfmm_tuner_input(const float* features, int order, int depth, int precision, float* row);
/* Proposes (order, depth, precision) with the smallest predicted time whose predicted
 * relative force error times 'margin' is within 'tol'.  GBFMM_ERR_UNSUPPORTED if no
 * candidate is predicted to meet it (the caller then keeps the plain FMM). */
int gbfmm_tuner_propose(gbfmm_mlp* m, const float* features, double tol, double margin, int* order, int* depth,
                        int* precision, float* pred_err, float* pred_ms);

/* Depth of the plain FMM for natoms bodies: 16-128 bodies per leaf. */
int gbfmm_plain_depth(int natoms);

/* The checked choice (no counterpart in the reference, which fixes P=10 and
 * depth 3, zeta_fmm_solver.cpp:10-11): statistics of the system on the device,
 * the network's proposal for 'tol' (gbfmm_tuner_propose with 'margin'), then a
 * check of the proposal's forces against the plain order-10 FP32 FMM of the
 * same configuration (the check solve), retried at one and two orders higher; an
 * accepted order is refined downwards (one order lower at the same depth and
 * precision, while the difference from the check solve stays within tol / margin, down to
 * order 4); when no candidate meets tol, or none is proposed, the plain FMM's
 * parameters are chosen (fallback = 1).  Host inputs; each solve runs through
 * gbfmm_execute. */
#define GBFMM_TUNER_MAX_CHECKS 8
typedef struct {
    int order, depth, precision;  /* the choice */
    int fallback;                 /* 1: the plain FMM */
    double diff_vs_plain;         /* relative RMS force difference of the choice from the check solve */
    int proposed_order, proposed_depth, proposed_precision;  /* the network's proposal (0 if none) */
    float pred_rel_force_err, pred_ms;
    int nchecks;                  /* checked candidates (orders check_order[k]) */
    int check_order[GBFMM_TUNER_MAX_CHECKS];
    double check_diff[GBFMM_TUNER_MAX_CHECKS];
} gbfmm_tuner_choice;
int gbfmm_tuner_choose(gbfmm_mlp* m, int natoms, const float* charges, const float* coords, const float* box,
                       int images, double tol, double margin, gbfmm_tuner_choice* out);

/* ---- tree build without allocation ---- */

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory at call time (an MD engine whose own pool reserved the GPU's memory at
 * start-up, or a time-stepping loop that must not call cudaMalloc because it can
 * synchronise the device): builds the same tree as gbfmm_execute
 * -- order[i] = input index of the body at sorted position i, leaf_offsets[k] =
 * first body of leaf k in BFS order, leaf_offsets[8^depth] = natoms -- using
 * only a fixed static device array for scratch.  Inputs and outputs are device
 * pointers: coords float[3*natoms], charges float[natoms], order int[natoms],
 * leaf_offsets int[8^depth + 1]; box float[9] on the host (cubic).
 * Limits: natoms <= GBFMM_NOALLOC_MAX_ATOMS and depth <= GBFMM_NOALLOC_MAX_DEPTH;
 * larger inputs return GBFMM_ERR_ARG.  The first call in each CUDA context of a
 * device looks up the array's device address (make it before any stream capture;
 * after cudaDeviceReset the next call looks it up again).  All calls share
 * the scratch: calls that overlap on the GPU race.  Asynchronous on 'stream';
 * non-finite coordinates are not reported (no host read-back). */
#define GBFMM_NOALLOC_MAX_ATOMS 65536
#define GBFMM_NOALLOC_MAX_DEPTH 4
int gbfmm_tree_build_noalloc(const void* coords, const void* charges, int natoms, const float* box, int max_depth,
                             void* order, void* leaf_offsets, void* stream);

/* ---- operator tables (host only, for tests) ---- */

/* Fills 'mat' (rows x cols, row-major, real (P+1)^2 representation in scaled
 * units) with one operator the device kernels apply.  kind: 0 M2M of child
 * octant 'index', 1 L2L of child octant 'index', 2 M2L class 'index', 3 the
 * periodic lattice operator.  Returns GBFMM_ERR_ARG for an unknown index. */
int gbfmm_debug_operator(int order, int images, int kind, int index, double* mat, int* dim, double* class_vec);
int gbfmm_debug_harmonics(int order, int kind, const double* d, double* out);
/* Runs the library's bounded mbarrier wait in a one-warp kernel on a barrier
 * that nothing completes (no copies or MMAs in flight), with a limit of 'polls'
 * polls.  Returns GBFMM_ERR_TIMEOUT when the wait gave up (the context stays
 * usable), as a step does when one of its bounded waits gives up. */
int gbfmm_debug_bounded_wait(unsigned polls, void* stream);

/* ---- autotuner (tile shapes) ----
 * gbfmm_autotune times whole steps (CUDA-graph replays, reps per candidate, each
 * after a 256 MB write that flushes L2; the buffer is allocated for the call) of
 * the given configuration for the P2P variants (0-14: warp-step shape 8 x 4,
 * 4 x 8 or 16 x 2 by variant % 3, one CTA per leaf or 2-5 resident CTAs per SM
 * by variant / 3; 15-16: 8 x 4 and 4 x 8 with up to 4 targets per thread, one
 * CTA per leaf) and, on the tensor-core
 * path, the M2L entry split (1, 2, 4, 8; 1 only on a deterministic handle)
 * together with the pipeline depth, then where the near field starts
 * (gbfmm_set_near_start), then the split, depth and P2P variant again at that
 * start, and keeps the fastest (best_ms: its step time; may be NULL).
 * Results are the same up to the order of floating-point additions.  No
 * reference counterpart: the reference's launch shapes are fixed
 * (gpu_solver.cu:221-248). */
int gbfmm_autotune(gbfmm_handle* h, const float* coords, const float* box, int reps, float* best_ms);
/* Where the near field starts in the step's graph: after the tree (0, the
 * default), after the P2M (1) or after the upper tree (2).  The near field runs
 * on a low-priority stream beside the far-field chain either way; starting it
 * later lets the far-field kernels with large shared memory take SMs before its
 * CTAs fill them.  Results do not depend on it; gbfmm_autotune searches it. */
int gbfmm_set_near_start(gbfmm_handle* h, int after);
int gbfmm_get_near_start(gbfmm_handle* h, int* after);
/* Programmatic dependent launches in the step (on by default): each kernel of the
 * far-field chain that follows another on the same stream may start while that
 * one finishes (it stages its constant operators meanwhile and waits for the
 * previous kernel's completion before it touches its data).  Off, every kernel
 * starts after the previous one ends.  Results do not depend on it. */
int gbfmm_set_launch_overlap(gbfmm_handle* h, int enable);
int gbfmm_get_launch_overlap(gbfmm_handle* h, int* enable);
int gbfmm_get_tuning(gbfmm_handle* h, int* p2p_variant, int* m2l_split, int* m2l_stages);
int gbfmm_set_tuning(gbfmm_handle* h, int p2p_variant, int m2l_split, int m2l_stages);

/* ---- batched solves ---- */

/* Many independent cubic systems solved as one batch through one captured
 * CUDA graph.  Host inputs: offsets[n_sys+1] into the concatenated coords
 * (3 floats per atom) and charges, boxes[n_sys] (cubic edge, nm), per-system
 * order and depth; flags as gbfmm_params.flags (GBFMM_FLAG_NO_GRAPH is
 * ignored: a batch always replays its graph).  Outputs (host): forces,
 * potentials, energies[n_sys]. */
typedef struct gbfmm_batch gbfmm_batch;
int gbfmm_batch_create(int n_sys, const int* atom_offsets, const int* orders, const int* depths, int images,
                       int precision, int flags, gbfmm_batch** out);
/* As gbfmm_batch_create, with each system's own M2L precision (precisions[n_sys],
 * GBFMM_PREC_*).  No reference counterpart (the reference solves one system). */
int gbfmm_batch_create_mixed(int n_sys, const int* atom_offsets, const int* orders, const int* depths,
                             const int* precisions, int images, int flags, gbfmm_batch** out);
int gbfmm_batch_execute(gbfmm_batch* b, const float* coords, const float* charges, const float* box_edges,
                        float* forces, float* potentials, double* energies);
/* Device-resident batch step, asynchronous on 'stream'.  It reads no device
 * status back: a system's errors (non-finite input, a bounded device wait that
 * gave up) are reported by gbfmm_batch_status, or by the next gbfmm_batch_execute. */
int gbfmm_batch_execute_device(gbfmm_batch* b, const void* d_coords, const void* d_charges,
                               const float* box_edges, void* stream);
/* Waits for the batch's last step and reports its systems' errors: GBFMM_ERR_COORD
 * (a non-finite coordinate or charge) or GBFMM_ERR_TIMEOUT (a bounded device
 * wait gave up); the flags and step counters are then cleared for the next step. */
int gbfmm_batch_status(gbfmm_batch* b);
int gbfmm_batch_device_outputs(gbfmm_batch* b, void** d_forces, void** d_potentials, void** d_energies);
/* Number of device kernels one batch step launches: each kind of kernel runs for
 * every system in one launch (one per expansion order or shared-memory size
 * where the kernel depends on them), the near fields in one persistent kernel. */
int gbfmm_batch_step_launches(gbfmm_batch* b, int* n);
int gbfmm_batch_destroy(gbfmm_batch* b);

/* Batch schedule: the far fields run as 'far_lanes' concurrent chains of
 * grouped launches (1..min(n_sys, 8); the expansion orders are spread over the
 * lanes, heaviest first), on streams of the greatest priority when far_prio is
 * non-zero, and the near-field kernel starts after the tree (near_after 0),
 * together with the M2L (1) or after it (2).  The results do not depend on the
 * schedule.  Default 1, 0, 0; gbfmm_batch_autotune searches it too. */
int gbfmm_batch_set_schedule(gbfmm_batch* b, int far_lanes, int far_prio, int near_after);
int gbfmm_batch_get_schedule(gbfmm_batch* b, int* far_lanes, int* far_prio, int* near_after);

/* Batch autotuner: times replays of the batch graph on the caller's device
 * inputs (as gbfmm_batch_execute_device; each after an L2 flush) for the near-field kernel's warp-step
 * shape (0: 8 targets x 4 source lanes, 1: 4 x 8, 2: 16 x 2, 3 and 4: 8 x 4 and
 * 4 x 8 with up to 4 targets per thread) and residency (2..5 resident CTAs
 * per SM walking the queue, or 0: one CTA per leaf), then, when
 * any system uses the tensor-core M2L, a batch-wide M2L entry split (1, 2, 4,
 * 8) and pipeline depth, then the schedule (gbfmm_batch_set_schedule: lanes
 * up to one per expansion order, their priority, near_after 0 or 1), and keeps
 * the fastest (best_ms: its step time).
 * m2l_split / m2l_stages 0 in get/set mean each system's own.  Results are the
 * same up to the order of floating-point additions.  No reference counterpart:
 * the reference solves one system per call with fixed launch shapes
 * (gpu_solver.cu:221-248). */
int gbfmm_batch_autotune(gbfmm_batch* b, const void* d_coords, const void* d_charges, const float* box_edges,
                         int reps, float* best_ms);
int gbfmm_batch_get_tuning(gbfmm_batch* b, int* p2p_shape, int* p2p_per_sm, int* m2l_split, int* m2l_stages);
int gbfmm_batch_set_tuning(gbfmm_batch* b, int p2p_shape, int p2p_per_sm, int m2l_split, int m2l_stages);

#ifdef __cplusplus
}
#endif
#endif /* GBFMM_H */
