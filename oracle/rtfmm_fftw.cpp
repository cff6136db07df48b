// Multidimensional real DFTs behind oracle/rtfmm_shim/fftw3.h (TEST
// INFRASTRUCTURE ONLY): the FFTW 3 calls of the reference's CPU FMM, computed
// from the DFT's definition as separable 1-D transforms with precomputed
// twiddle tables (O(n^2) per 1-D transform: the convolution grids of that FMM
// are small, 2P-1 points per edge).  Conventions of FFTW: forward sign -1, the
// inverse unnormalised, r2c/c2r keep the last dimension's n/2+1 bins, row-major,
// and execute calls on new arrays are reentrant (scratch on the caller's stack
// frame).
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "rtfmm_shim/fftw3.h"

namespace {

using cd = std::complex<double>;

struct Plan {
    bool r2c = true;
    int n[3] = {1, 1, 1};
    int howmany = 1;
    long idist = 0, odist = 0;  // in elements of the input / output type
    double* rin = nullptr;
    fftw_complex* cin = nullptr;
    double* rout = nullptr;
    fftw_complex* cout = nullptr;
    std::vector<cd> w[3];        // w[d][k] = exp(-2 pi i k / n[d])
};

void twiddles(Plan& p)
{
    for (int d = 0; d < 3; d++) {
        p.w[d].resize(p.n[d]);
        for (int k = 0; k < p.n[d]; k++) {
            const double a = -2.0 * M_PI * k / p.n[d];
            p.w[d][k] = cd(std::cos(a), std::sin(a));
        }
    }
}

// In-place 1-D complex DFT of the n values at x[0], x[s], ..., sign -1 (forward)
// or +1 (inverse, w conjugated).
void dft1(cd* x, long s, int n, const std::vector<cd>& w, bool inverse, cd* tmp)
{
    for (int k = 0; k < n; k++) {
        cd acc(0.0, 0.0);
        int idx = 0;
        for (int j = 0; j < n; j++) {
            const cd t = inverse ? std::conj(w[idx]) : w[idx];
            acc += x[j * s] * t;
            idx += k;
            if (idx >= n) idx -= n;
        }
        tmp[k] = acc;
    }
    for (int k = 0; k < n; k++) x[k * s] = tmp[k];
}

void r2c_one(const Plan& p, const double* in, cd* out)
{
    const int n0 = p.n[0], n1 = p.n[1], n2 = p.n[2], h = n2 / 2 + 1;
    std::vector<cd> tmp(std::max(n0, std::max(n1, n2)));
    // last dimension: real input, the first h bins
    for (long r = 0; r < (long)n0 * n1; r++) {
        const double* x = in + r * n2;
        cd* y = out + r * h;
        for (int k = 0; k < h; k++) {
            cd acc(0.0, 0.0);
            int idx = 0;
            for (int j = 0; j < n2; j++) {
                acc += x[j] * p.w[2][idx];
                idx += k;
                if (idx >= n2) idx -= n2;
            }
            y[k] = acc;
        }
    }
    for (int i0 = 0; i0 < n0; i0++)
        for (int k = 0; k < h; k++) dft1(out + (long)i0 * n1 * h + k, h, n1, p.w[1], false, tmp.data());
    for (int i1 = 0; i1 < n1; i1++)
        for (int k = 0; k < h; k++) dft1(out + (long)i1 * h + k, (long)n1 * h, n0, p.w[0], false, tmp.data());
}

void c2r_one(const Plan& p, const cd* in, double* out)
{
    const int n0 = p.n[0], n1 = p.n[1], n2 = p.n[2], h = n2 / 2 + 1;
    std::vector<cd> z(in, in + (long)n0 * n1 * h);
    std::vector<cd> tmp(std::max(n0, std::max(n1, n2)));
    for (int i1 = 0; i1 < n1; i1++)
        for (int k = 0; k < h; k++) dft1(z.data() + (long)i1 * h + k, (long)n1 * h, n0, p.w[0], true, tmp.data());
    for (int i0 = 0; i0 < n0; i0++)
        for (int k = 0; k < h; k++) dft1(z.data() + (long)i0 * n1 * h + k, h, n1, p.w[1], true, tmp.data());
    // last dimension: the half spectrum of a real sequence (Hermitian extension)
    for (long r = 0; r < (long)n0 * n1; r++) {
        const cd* y = z.data() + r * h;
        double* x = out + r * n2;
        for (int j = 0; j < n2; j++) {
            double acc = y[0].real();
            int idx = j;
            for (int k = 1; k < h; k++) {
                const cd t = y[k] * std::conj(p.w[2][idx]);
                acc += (2 * k == n2) ? t.real() : 2.0 * t.real();
                idx += j;
                if (idx >= n2) idx -= n2;
            }
            x[j] = acc;
        }
    }
}

Plan* make(bool r2c, int rank, const int* n, int howmany)
{
    if (rank != 3) return nullptr;
    Plan* p = new Plan();
    p->r2c = r2c;
    for (int d = 0; d < 3; d++) p->n[d] = n[d];
    p->howmany = howmany;
    twiddles(*p);
    return p;
}

void run(const Plan& p, const double* rin, const fftw_complex* cin, double* rout, fftw_complex* cout)
{
    const long nr = (long)p.n[0] * p.n[1] * p.n[2], nc = (long)p.n[0] * p.n[1] * (p.n[2] / 2 + 1);
    const long id = p.idist ? p.idist : (p.r2c ? nr : nc), od = p.odist ? p.odist : (p.r2c ? nc : nr);
    for (int b = 0; b < p.howmany; b++) {
        if (p.r2c)
            r2c_one(p, rin + b * id, reinterpret_cast<cd*>(cout + b * od));
        else
            c2r_one(p, reinterpret_cast<const cd*>(cin + b * id), rout + b * od);
    }
}

}  // namespace

extern "C" {

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double* in, fftw_complex* out, unsigned)
{
    const int n[3] = {n0, n1, n2};
    Plan* p = make(true, 3, n, 1);
    p->rin = in;
    p->cout = out;
    return reinterpret_cast<fftw_plan>(p);
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex* in, double* out, unsigned)
{
    const int n[3] = {n0, n1, n2};
    Plan* p = make(false, 3, n, 1);
    p->cin = in;
    p->rout = out;
    return reinterpret_cast<fftw_plan>(p);
}

fftw_plan fftw_plan_many_dft_r2c(int rank, const int* n, int howmany, double* in, const int*, int, int idist,
                                 fftw_complex* out, const int*, int, int odist, unsigned)
{
    Plan* p = make(true, rank, n, howmany);
    if (!p) return nullptr;
    p->rin = in;
    p->cout = out;
    p->idist = idist;
    p->odist = odist;
    return reinterpret_cast<fftw_plan>(p);
}

fftw_plan fftw_plan_many_dft_c2r(int rank, const int* n, int howmany, fftw_complex* in, const int*, int, int idist,
                                 double* out, const int*, int, int odist, unsigned)
{
    Plan* p = make(false, rank, n, howmany);
    if (!p) return nullptr;
    p->cin = in;
    p->rout = out;
    p->idist = idist;
    p->odist = odist;
    return reinterpret_cast<fftw_plan>(p);
}

void fftw_execute(const fftw_plan p)
{
    const Plan* q = reinterpret_cast<const Plan*>(p);
    run(*q, q->rin, q->cin, q->rout, q->cout);
}

void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out)
{
    run(*reinterpret_cast<const Plan*>(p), in, nullptr, nullptr, out);
}

void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex* in, double* out)
{
    run(*reinterpret_cast<const Plan*>(p), nullptr, in, out, nullptr);
}

void fftw_destroy_plan(fftw_plan p) { delete reinterpret_cast<Plan*>(p); }

}  // extern "C"
