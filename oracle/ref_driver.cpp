// Driver around the reference's own zeta_fmm tree and traverser (TEST INFRASTRUCTURE ONLY).
//
// Compiled by oracle/ref_build.sh together with the UNMODIFIED reference sources
//   src/gromacs/zeta_fmm/tree.cpp       (CompleteBalancedOctree::build, :13-99)
//   src/gromacs/zeta_fmm/traverser.cpp  (NearFieldSelector, Traverser, :9-214)
// into oracle/_ref/libzetaref.so.  It runs the reference exactly as
// GPUSolver::prepare_maps does (src/gromacs/zeta_fmm/gpu_solver.cu:36-61: build,
// build_reg with rega=0, MAC selector with scale theta, traverse) and exposes the
// resulting cells, body order and P2P/M2L maps through a C ABI so that golden
// fixtures can be generated from the reference itself.
#include <cstring>
#include <vector>

#include "traverser.h"
#include "tree.h"

namespace {
std::vector<zeta_fmm::Cell3> g_cells;
std::vector<int> g_order;
zeta_fmm::Traverser::CellMap g_p2p, g_m2l;
}  // namespace

extern "C" int zref_run(int n, const double* xyz, double box_r, const double* center, int max_depth, int images,
                        double cycle, double theta)
{
    std::vector<zeta_fmm::Body3> bodies(n);
    for (int i = 0; i < n; i++) {
        bodies[i].idx = i;
        bodies[i].loc = zeta_fmm::vec3r(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    }
    zeta_fmm::CompleteBalancedOctree tree;
    tree.build(bodies, box_r, zeta_fmm::vec3r(center[0], center[1], center[2]), max_depth);
    tree.build_reg(bodies, 0.0, max_depth, cycle);
    zeta_fmm::NearFieldSelector sel(zeta_fmm::NearFieldSelector::SelectorType::MAC, theta);
    zeta_fmm::Traverser trav;
    trav.traverse(tree, sel, images, cycle);
    g_cells = trav.get_cells();
    g_p2p = trav.get_p2p_map();
    g_m2l = trav.get_m2l_map();
    g_order.resize(n);
    for (int i = 0; i < n; i++) g_order[i] = bodies[i].idx;
    return (int)g_cells.size();
}

extern "C" void zref_cells(int* depth, double* r, double* center, int* child_off, int* child_num, int* body_off,
                           int* body_num)
{
    for (size_t i = 0; i < g_cells.size(); i++) {
        const zeta_fmm::Cell3& c = g_cells[i];
        depth[i] = c.depth;
        r[i] = c.r;
        center[3 * i] = c.center[0];
        center[3 * i + 1] = c.center[1];
        center[3 * i + 2] = c.center[2];
        child_off[i] = c.child_info.offset;
        child_num[i] = c.child_info.number;
        body_off[i] = c.body_info.offset;
        body_num[i] = c.body_info.number;
    }
}

extern "C" void zref_order(int* idx) { std::memcpy(idx, g_order.data(), sizeof(int) * g_order.size()); }

extern "C" long zref_nlist(int which)
{
    const zeta_fmm::Traverser::CellMap& m = which == 0 ? g_p2p : g_m2l;
    long n = 0;
    for (const auto& kv : m) n += (long)kv.second.size();
    return n;
}

// Flattened in std::map iteration order: ascending target, append order within a target.
extern "C" void zref_list(int which, int* tgt, int* src, double* off)
{
    const zeta_fmm::Traverser::CellMap& m = which == 0 ? g_p2p : g_m2l;
    long e = 0;
    for (const auto& kv : m) {
        for (const auto& io : kv.second) {
            tgt[e] = kv.first;
            src[e] = io.idx;
            off[3 * e] = io.offset.x;
            off[3 * e + 1] = io.offset.y;
            off[3 * e + 2] = io.offset.z;
            e++;
        }
    }
}
