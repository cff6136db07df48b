// Test stand-in for the parts of GROMACS' gromacs/math/vectypes.h and
// gromacs/utility/arrayref.h that the drop-in adapter uses (same names and
// layouts: RVec is three floats, matrix float[3][3], ArrayRef a pointer and a
// size).  Only for compiling and running the adapter without a GROMACS tree.
#pragma once
#include <cstddef>

typedef float real;
#define DIM 3
typedef real matrix[DIM][DIM];

namespace gmx
{
class RVec
{
public:
    RVec() : x_{0, 0, 0} {}
    RVec(real x, real y, real z) : x_{x, y, z} {}
    real& operator[](int d) { return x_[d]; }
    const real& operator[](int d) const { return x_[d]; }
    real* as_vec() { return x_; }
    const real* as_vec() const { return x_; }

private:
    real x_[DIM];
};
static_assert(sizeof(RVec) == 3 * sizeof(real), "RVec is packed");

template <typename T>
class ArrayRef
{
public:
    ArrayRef() = default;
    ArrayRef(T* begin, std::size_t n) : p_(begin), n_(n) {}
    template <typename U>
    ArrayRef(const ArrayRef<U>& o) : p_(o.data()), n_(o.size())
    {
    }
    T* data() const { return p_; }
    std::size_t size() const { return n_; }
    T& operator[](std::size_t i) const { return p_[i]; }
    T* begin() const { return p_; }
    T* end() const { return p_ + n_; }

private:
    T* p_ = nullptr;
    std::size_t n_ = 0;
};
}  // namespace gmx
