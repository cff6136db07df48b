// Test stand-in for GROMACS' gmx::ForceWithVirial: the force buffer and the
// virial contributions of force providers that compute their own virial
// (same member names and signatures as gromacs/mdtypes/forceoutput.h).
#pragma once
#include "gromacs/math/vectypes.h"

namespace gmx
{
class ForceWithVirial
{
public:
    ForceWithVirial(ArrayRef<RVec> f, bool computeVirial) : force_(f), computeVirial_(computeVirial) {}
    // Adds a virial contribution, -1/2 sum r (x) F convention (kJ/mol).
    void addVirialContribution(const matrix virial)
    {
        if (!computeVirial_) return;
        for (int i = 0; i < DIM; i++)
            for (int j = 0; j < DIM; j++) virial_[i][j] += virial[i][j];
        haveVirialContributions_ = true;
    }
    bool haveVirialContributions() const { return haveVirialContributions_; }
    double virial(int i, int j) const { return virial_[i][j]; }
    const ArrayRef<RVec> force_;
    const bool computeVirial_;

private:
    bool haveVirialContributions_ = false;
    double virial_[DIM][DIM] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
};
}  // namespace gmx
