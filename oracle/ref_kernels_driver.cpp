// Runs the reference's own FP64 FMM kernels on the host (TEST INFRASTRUCTURE ONLY).
//
// Linked by oracle/ref_build.sh with the UNMODIFIED kernels of
// src/gromacs/zeta_fmm/kernel.cu (everything before GPUKernel::GPUKernel(),
// compiled as host code through oracle/ref_cuda_shim.h) and the reference's
// tree.cpp / traverser.cpp.  zref_solve follows GPUSolver::solve
// (gpu_solver.cu:63-260) for rega = 0:
//   - build, build_reg(0), MAC 0.4 traversal (gpu_solver.cu:36-61);
//   - leaf list = cells of the deepest level of depth_map (:281-301), branch cells
//     per level from the deepest branch level to 0 and image cells from the
//     depth_map in reverse order (:118-147), P2P/M2L matrices in std::map order
//     (:149-219);
//   - the launch sequence of GPUKernel::solve (kernel.cu:815-913): p2m, m2m per
//     level, m2m_image, m2l, p2p, l2l per level in reverse, l2p; each launch of
//     <<<grid, block>>> becomes a loop over blocks and threads;
//   - the unit conversion of gpu_solver.cu:250-256 (p *= ke, f *= -q ke).
// Outputs are in input order (Body3::idx), before the dipole correction of
// solver.cpp.
#include <cstring>
#include <map>
#include <vector>

#include "kernel.h"
#include "traverser.h"
#include "tree.h"

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;

// the kernels of kernel.cu (global namespace)
void p2m(zeta_fmm::Body3*, zeta_fmm::Cell3*, int*, int, zeta_fmm::complex*);
void m2m(zeta_fmm::Cell3*, int*, int, int, zeta_fmm::complex*);
void m2m_image(zeta_fmm::Cell3*, int*, int, int, zeta_fmm::complex*, zeta_fmm::real);
void m2l(zeta_fmm::Cell3*, int*, zeta_fmm::Offset3rPadding*, int, int, zeta_fmm::complex*, zeta_fmm::complex*);
void p2p(zeta_fmm::Body3*, zeta_fmm::Cell3*, int*, zeta_fmm::Offset3rPadding*, int);
void l2l(zeta_fmm::Cell3*, int*, int, int, zeta_fmm::complex*);
void l2p(zeta_fmm::Body3*, zeta_fmm::Cell3*, int*, int, zeta_fmm::complex*);

namespace {

constexpr double KE = 138.935457833;  // gmx::c_one4PiEps0 (units.h)

template <typename F>
void launch(unsigned grid, unsigned block, F&& kernel)
{
    gridDim = dim3(grid, 1, 1);
    blockDim = dim3(block, 1, 1);
    for (unsigned b = 0; b < grid; b++) {
        blockIdx = make_uint3(b, 0, 0);
        for (unsigned t = 0; t < block; t++) {
            threadIdx = make_uint3(t, 0, 0);
            kernel();
        }
    }
}

// P2P / M2L matrix of gpu_solver.cu:149-219: per target row [target, count,
// sources..., padding] and the periodic offsets of the sources.
void pack(const zeta_fmm::Traverser::CellMap& map, std::vector<int>& mat, std::vector<zeta_fmm::Offset3rPadding>& off,
          int& rows, int& cols)
{
    int maxs = 0;
    for (const auto& kv : map) maxs = std::max(maxs, (int)kv.second.size());
    rows = (int)map.size();
    cols = maxs + 2;
    mat.assign((size_t)rows * cols, 0);
    off.assign((size_t)rows * (cols - 2), zeta_fmm::Offset3rPadding{0, 0, 0, 0});
    int i = 0;
    for (const auto& kv : map) {
        mat[(size_t)i * cols] = kv.first;
        mat[(size_t)i * cols + 1] = (int)kv.second.size();
        for (size_t j = 0; j < kv.second.size(); j++) {
            mat[(size_t)i * cols + 2 + j] = kv.second[j].idx;
            zeta_fmm::Offset3rPadding o;
            o.x = kv.second[j].offset.x;
            o.y = kv.second[j].offset.y;
            o.z = kv.second[j].offset.z;
            o.padding = 0;
            off[(size_t)i * (cols - 2) + j] = o;
        }
        i++;
    }
}

}  // namespace

// FP64 potentials (kJ/mol/e) and forces (kJ/mol/nm) of the reference's GPU
// kernels, input order, without the dipole correction.  Returns 0 on success.
extern "C" int zref_solve(int n, const double* xyz, const double* q, double cycle, int P, int max_depth, int images,
                          double* pot, double* force)
{
    if (n <= 0 || P < 1 || P > 20 || max_depth < 1) return -1;
    std::vector<zeta_fmm::Body3> bodies(n);
    for (int i = 0; i < n; i++) {
        bodies[i].idx = i;
        bodies[i].q = q[i];
        bodies[i].p = 0;
        bodies[i].f = zeta_fmm::vec3r(0, 0, 0);
        bodies[i].loc = zeta_fmm::vec3r(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    }
    const double box_r = cycle / 2;
    zeta_fmm::CompleteBalancedOctree tree;
    tree.build(bodies, box_r, zeta_fmm::vec3r(box_r, box_r, box_r), max_depth);
    tree.build_reg(bodies, 0.0, max_depth, cycle);
    zeta_fmm::NearFieldSelector sel(zeta_fmm::NearFieldSelector::SelectorType::MAC, 0.4);
    zeta_fmm::Traverser trav;
    trav.traverse(tree, sel, images, cycle);
    std::vector<zeta_fmm::Cell3> cells = trav.get_cells();
    zeta_fmm::Traverser::CellMap depth_map = trav.get_depth_map();
    zeta_fmm::Traverser::CellMap p2p_map = trav.get_p2p_map();
    zeta_fmm::Traverser::CellMap m2l_map = trav.get_m2l_map();

    int real_max_depth = 0;
    for (const auto& kv : depth_map) real_max_depth = std::max(real_max_depth, kv.first);
    std::vector<int> leaves;
    for (const auto& c : depth_map[real_max_depth]) leaves.push_back(c.idx);
    std::vector<int> branch;
    std::vector<zeta_fmm::OffsetAndNumber> level_infos;
    int level_offset = 0;
    for (auto it = depth_map.rbegin(); it != depth_map.rend(); ++it) {
        if (it->first == real_max_depth || it->first < 0) continue;
        level_infos.push_back(zeta_fmm::OffsetAndNumber(level_offset, (int)it->second.size()));
        for (const auto& c : it->second) branch.push_back(c.idx);
        level_offset += (int)it->second.size();
    }
    std::vector<int> img;
    for (auto it = depth_map.rbegin(); it != depth_map.rend(); ++it)
        if (it->first < 0) img.push_back(it->second[0].idx);
    std::vector<int> p2p_mat, m2l_mat;
    std::vector<zeta_fmm::Offset3rPadding> p2p_off, m2l_off;
    int p2p_rows, p2p_cols, m2l_rows, m2l_cols;
    pack(p2p_map, p2p_mat, p2p_off, p2p_rows, p2p_cols);
    pack(m2l_map, m2l_mat, m2l_off, m2l_rows, m2l_cols);

    const int np = get_pole_size_eachcell(P);
    std::vector<zeta_fmm::complex> Ms((size_t)cells.size() * np), Ls((size_t)cells.size() * np);
    for (auto& c : Ms) c.rel = c.img = 0;
    for (auto& c : Ls) c.rel = c.img = 0;
    zeta_fmm::Body3* B = bodies.data();
    zeta_fmm::Cell3* C = cells.data();

    launch((unsigned)leaves.size(), 1, [&] { p2m(B, C, leaves.data(), P, Ms.data()); });
    for (const auto& on : level_infos)
        launch((unsigned)on.number, 1, [&] { m2m(C, branch.data(), on.offset, P, Ms.data()); });
    double cyc = cycle;
    for (int i = 0; i + 1 < (int)img.size(); i++) {
        launch(1, 1, [&] { m2m_image(C, img.data(), i, P, Ms.data(), cyc); });
        cyc *= 3;
    }
    if (m2l_rows > 0)
        launch((unsigned)m2l_rows, 1,
               [&] { m2l(C, m2l_mat.data(), m2l_off.data(), m2l_cols, P, Ms.data(), Ls.data()); });
    if (p2p_rows > 0)
        launch((unsigned)p2p_rows, 64, [&] { p2p(B, C, p2p_mat.data(), p2p_off.data(), p2p_cols); });
    for (int i = (int)level_infos.size() - 1; i >= 0; i--) {
        const zeta_fmm::OffsetAndNumber on = level_infos[i];
        launch((unsigned)on.number, 1, [&] { l2l(C, branch.data(), on.offset, P, Ls.data()); });
    }
    launch((unsigned)leaves.size(), 1, [&] { l2p(B, C, leaves.data(), P, Ls.data()); });

    for (const zeta_fmm::Body3& b : bodies) {
        pot[b.idx] = b.p * KE;
        for (int d = 0; d < 3; d++) force[3 * b.idx + d] = b.f[d] * (-b.q * KE);
    }
    return 0;
}
