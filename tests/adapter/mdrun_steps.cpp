// Drives the drop-in adapter (gromacs-fmm_gb300/adapter/gbfmm_solver.h) the way
// mdrun drives a coulomb_solver::BaseSolver (SolverExecuter, sim_util.cpp and
// md.cpp of the fork): construct once, then per step set_parameter, execute,
// add_force into the step's force buffer, get_energy; compare_forces at the end.
//
// usage: mdrun_steps in.bin out.bin order depth images [tol weights]
//   in.bin : int32 natoms, int32 nsteps, float box[9], float q[natoms],
//            float x[nsteps][natoms][3]
//   out.bin: per step float f[natoms][3] (added to a buffer of ones), double energy,
//            double virial[3][3] (the step's ForceWithVirial computes the virial)
//   order 0: the learned tuner's checked choice for the force tolerance 'tol'
//   (weights file 'weights'), printed as "choice order depth precision fallback"
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <vector>

#include "gbfmm_solver.h"

int main(int argc, char** argv)
{
    if (argc != 6 && argc != 8) {
        std::fprintf(stderr, "usage: %s in.bin out.bin order depth images [tol weights]\n", argv[0]);
        return 2;
    }
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int n = 0, nsteps = 0;
    matrix box;
    if (std::fread(&n, sizeof(int), 1, in) != 1 || std::fread(&nsteps, sizeof(int), 1, in) != 1 ||
        std::fread(&box[0][0], sizeof(float), 9, in) != 9)
        return 2;
    std::vector<real> q(n);
    std::vector<gmx::RVec> x((size_t)n * nsteps);
    if (std::fread(q.data(), sizeof(float), n, in) != (size_t)n ||
        std::fread(x.data(), sizeof(float), 3 * (size_t)n * nsteps, in) != 3 * (size_t)n * nsteps)
        return 2;
    std::fclose(in);
    FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    try {
        t_mdatoms md;
        md.homenr = n;
        md.chargeA = gmx::ArrayRef<real>(q.data(), n);
        md.chargeB = gmx::ArrayRef<real>(q.data(), n);
        gbfmm_params p;
        gbfmm_params_default(&p);
        p.order = std::atoi(argv[3]);
        p.max_depth = std::atoi(argv[4]);
        p.images = std::atoi(argv[5]);
        const bool tuned = p.order == 0;
        coulomb_solver::GbFmmSolver solver = tuned ? coulomb_solver::GbFmmSolver(stdout, md, std::atof(argv[6]), argv[7])
                                                   : coulomb_solver::GbFmmSolver(stdout, md, &p);
        coulomb_solver::BaseSolver& s = solver;  // mdrun holds the base class
        std::vector<gmx::RVec> f(n);
        for (int step = 0; step < nsteps; step++) {
            s.set_parameter(md);
            s.execute(gmx::ArrayRef<const gmx::RVec>(x.data() + (size_t)step * n, n), box, 0, 0);
            for (auto& v : f) v = gmx::RVec(1.f, 1.f, 1.f);
            gmx::ForceWithVirial fv(gmx::ArrayRef<gmx::RVec>(f.data(), n), true);
            s.add_force(&fv);
            const coulomb_solver::Energy e = s.get_energy();
            std::fwrite(f.data(), sizeof(float), 3 * (size_t)n, out);
            std::fwrite(&e.coulomb_energy, sizeof(double), 1, out);
            double vir[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) vir[3 * i + j] = fv.virial(i, j);
            std::fwrite(vir, sizeof(double), 9, out);
        }
        if (tuned)
            std::printf("choice %d %d %d %d\n", solver.choice().order, solver.choice().depth,
                        solver.choice().precision, solver.choice().fallback);
        for (auto& v : f) v = gmx::RVec(v[0] - 1.f, v[1] - 1.f, v[2] - 1.f);
        s.compare_forces(gmx::ArrayRef<gmx::RVec>(f.data(), n));
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        std::fclose(out);
        return 1;
    }
    std::fclose(out);
    return 0;
}
