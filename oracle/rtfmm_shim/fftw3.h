/* The subset of the FFTW 3 interface that the reference's CPU FMM uses
 * (src/gromacs/rtfmm/kernel.cpp: 3-D real-to-complex and complex-to-real plans,
 * single and batched, executed on their own or on new arrays).  TEST
 * INFRASTRUCTURE ONLY: it lets the reference's sources compile where FFTW is not
 * installed.  Same conventions as FFTW: forward sign -1, unnormalised inverse,
 * r2c output n0 x n1 x (n2/2 + 1), row-major.  Implemented by
 * oracle/rtfmm_fftw.cpp as separable DFTs with precomputed twiddles (FFTW's
 * own algorithms are not used). */
#ifndef GBFMM_FFTW_SUBSET_H
#define GBFMM_FFTW_SUBSET_H
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef struct fftw_plan_s* fftw_plan;
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_MEASURE (0U)
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex* in, double* out, unsigned flags);
fftw_plan fftw_plan_many_dft_r2c(int rank, const int* n, int howmany, double* in, const int* inembed, int istride,
                                 int idist, fftw_complex* out, const int* onembed, int ostride, int odist,
                                 unsigned flags);
fftw_plan fftw_plan_many_dft_c2r(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed,
                                 int istride, int idist, double* out, const int* onembed, int ostride, int odist,
                                 unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex* in, double* out);
void fftw_destroy_plan(fftw_plan p);
#ifdef __cplusplus
}
#endif
#endif
