// Test stand-in for the members of GROMACS' t_mdatoms that the solvers read.
#pragma once
#include "gromacs/math/vectypes.h"

struct t_mdatoms
{
    int homenr = 0;
    gmx::ArrayRef<real> chargeA;
    gmx::ArrayRef<real> chargeB;
};
