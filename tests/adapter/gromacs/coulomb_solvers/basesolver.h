// Test stand-in for the fork's coulomb_solver::BaseSolver interface
// (src/gromacs/coulomb_solvers/basesolver.h:10-90): the same class names,
// virtual methods and protected members, written here so that the adapter
// compiles and runs without a GROMACS tree.
#pragma once
#include <cstdio>

#include "gromacs/math/vectypes.h"
#include "gromacs/mdtypes/forceoutput.h"
#include "gromacs/mdtypes/mdatom.h"

namespace coulomb_solver
{
class Energy
{
public:
    double coulomb_energy = 0, lj_energy = 0, potential_energy = 0, kinetic_energy = 0, total_energy = 0,
           conserved_energy = 0;
};

class BaseSolver
{
public:
    BaseSolver(FILE* f, const t_mdatoms& md)
    {
        fplog = f;
        set_parameter(md);
    }
    virtual ~BaseSolver() = default;
    virtual void set_parameter(const t_mdatoms& md)
    {
        natoms = md.homenr;
        chargeA_ = md.chargeA;
        chargeB_ = md.chargeB;
    }
    virtual void execute(gmx::ArrayRef<const gmx::RVec> coord, const matrix box, int verbose = 0, int dummy = 0) = 0;
    virtual void add_force(gmx::ForceWithVirial* forcewithvirial) = 0;
    virtual Energy get_energy() = 0;
    virtual void compare_forces(const gmx::ArrayRef<gmx::RVec>& fs) = 0;

protected:
    FILE* fplog = nullptr;
    int natoms = 0;
    gmx::ArrayRef<const float> chargeA_;
    gmx::ArrayRef<const float> chargeB_;
};
}  // namespace coulomb_solver
