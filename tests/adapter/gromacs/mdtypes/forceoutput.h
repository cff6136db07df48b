// Test stand-in for the force buffer of GROMACS' gmx::ForceWithVirial.
#pragma once
#include "gromacs/math/vectypes.h"

namespace gmx
{
class ForceWithVirial
{
public:
    explicit ForceWithVirial(ArrayRef<RVec> f) : force_(f) {}
    const ArrayRef<RVec> force_;
};
}  // namespace gmx
