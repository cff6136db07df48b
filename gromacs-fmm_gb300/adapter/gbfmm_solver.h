// The GROMACS-side drop-in: a coulomb_solver::BaseSolver that forwards to the
// C ABI of libgbfmm (include/gbfmm.h).  A maintainer copies this file to
// src/gromacs/coulomb_solvers/gbfmm_solver.h of the fork, adds GBFMM to
// SolverExecuter::SolverType (executer.h:30-35) with a branch in set_solver
// (executer.h:37-60), and passes SolverType::GBFMM in md.cpp:852.
//
// Mirrors zeta_fmm::ZetaFmmSolver (src/gromacs/zeta_fmm/zeta_fmm_solver.cpp),
// with these differences: the device state lives for the solver's lifetime
// (the reference allocates and frees it inside every execute); get_energy
// returns 0.5 * sum(q * phi) (the reference's is a stub, :109-115); add_force
// also adds the Coulomb virial on the steps mdrun computes one (the reference
// adds none, :66-76); errors throw instead of exit(); and, given a
// force-error tolerance instead of fixed parameters, the solver takes the
// learned tuner's checked choice of order, depth and M2L precision.
#pragma once

#include <cstdio>
#include <stdexcept>
#include <string>

#include "gbfmm.h"
#include "gromacs/coulomb_solvers/basesolver.h"

namespace coulomb_solver
{
class GbFmmSolver : public BaseSolver
{
public:
    // The reference's constants (zeta_fmm_solver.cpp:6-14): order 10, depth 3,
    // 4 images; params may override them (gbfmm_params_default fills the rest).
    GbFmmSolver(FILE* f, const t_mdatoms& md, const gbfmm_params* params = nullptr) : BaseSolver(f, md)
    {
        gbfmm_params p;
        if (params) p = *params;
        else gbfmm_params_default(&p);
        create(p);
    }

    // Learned parameters: at the first execute, the tuner network (weights file
    // of gromacs-fmm_gb300/tuner_weights.bin) proposes order, depth and M2L
    // precision for the relative force-error tolerance 'force_tol', checked
    // against the plain order-10 FMM of that configuration (gbfmm_tuner_choose,
    // which falls back to the plain FMM).
    GbFmmSolver(FILE* f, const t_mdatoms& md, double force_tol, const char* weights) :
        BaseSolver(f, md), tol_(force_tol), weights_(weights)
    {
    }
    ~GbFmmSolver() override
    {
        if (h_) gbfmm_destroy(h_);
    }
    GbFmmSolver(const GbFmmSolver&) = delete;  // owns the library handle
    GbFmmSolver& operator=(const GbFmmSolver&) = delete;

    // The tuner's choice (valid after the first execute of a tolerance-driven solver).
    const gbfmm_tuner_choice& choice() const { return choice_; }

    // basesolver.h:56-61.  The library copies the charges; mdrun calls this
    // every step (md.cpp:1252), so they are re-sent.
    void set_parameter(const t_mdatoms& md) override
    {
        BaseSolver::set_parameter(md);
        if (h_) check(gbfmm_set_charges(h_, natoms, chargeA_.data()));
    }

    // zeta_fmm_solver.cpp:16-64: RVec is float[3] and matrix float[3][3], so the
    // pointers pass straight through.
    void execute(gmx::ArrayRef<const gmx::RVec> coord, const matrix box, int verbose = 0, int = 0) override
    {
        if (!h_) choose(coord.data()[0].as_vec(), &box[0][0]);
        check(gbfmm_execute(h_, coord.data()[0].as_vec(), &box[0][0], verbose));
    }

    // zeta_fmm_solver.cpp:66-76: accumulates into the force buffer; on the steps
    // mdrun computes the virial (computeVirial_), also the Coulomb virial
    // -1/2 sum r_ij (x) F_ij of the lattice sum (gbfmm_get_virial), which a
    // ForceWithVirial provider must add itself (sim_util.cpp:2085).
    void add_force(gmx::ForceWithVirial* fv) override
    {
        check(gbfmm_add_forces(h_, fv->force_.data()[0].as_vec()));
        if (fv->computeVirial_) {
            double v[9];
            check(gbfmm_get_virial(h_, v));
            matrix m;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) m[i][j] = (real)v[3 * i + j];
            fv->addVirialContribution(m);
        }
    }

    Energy get_energy() override
    {
        Energy e;
        check(gbfmm_get_energy(h_, &e.coulomb_energy));
        return e;
    }

    // zeta_fmm_solver.cpp:78-107
    void compare_forces(const gmx::ArrayRef<gmx::RVec>& fs) override
    {
        double l2f = 0;
        if (gbfmm_compare_forces(h_, fs.data()[0].as_vec(), &l2f) != GBFMM_OK) std::fprintf(stderr, "have nan!\n");
        std::printf("L2f = %.8f\n", l2f);
    }

private:
    static void check(int rc)
    {
        if (rc != GBFMM_OK)
            throw std::runtime_error(std::string(gbfmm_status_string(rc)) + ": " + gbfmm_last_error());
    }
    void create(const gbfmm_params& p)
    {
        check(gbfmm_create(&p, natoms, &h_));
        check(gbfmm_set_charges(h_, natoms, chargeA_.data()));
    }
    void choose(const float* x, const float* box)
    {
        gbfmm_mlp* m = nullptr;
        check(gbfmm_mlp_load(weights_.c_str(), &m));
        const int rc = gbfmm_tuner_choose(m, natoms, chargeA_.data(), x, box, 4, tol_, 1.5, &choice_);
        gbfmm_mlp_destroy(m);
        check(rc);
        gbfmm_params p;
        gbfmm_params_default(&p);
        p.order = choice_.order;
        p.max_depth = choice_.depth;
        p.precision = choice_.precision;
        create(p);
        if (fplog)
            std::fprintf(fplog, "gbfmm: order %d, depth %d, precision %d for force tolerance %g%s\n", choice_.order,
                         choice_.depth, choice_.precision, tol_, choice_.fallback ? " (plain FMM)" : "");
    }
    gbfmm_handle* h_ = nullptr;
    double tol_ = 0;
    std::string weights_;
    gbfmm_tuner_choice choice_{};
};
}  // namespace coulomb_solver
