// dgesvd_ for the reference's CPU FMM (TEST INFRASTRUCTURE ONLY): forwarded to
// the LAPACK routine of the OpenBLAS that scipy bundles (exported as
// scipy_dgesvd_), which src/gromacs/rtfmm/mathfunc.cpp:95-98 calls.
extern "C" {
void scipy_dgesvd_(char* jobu, char* jobvt, int* m, int* n, double* a, int* lda, double* s, double* u, int* ldu,
                   double* vt, int* ldvt, double* work, int* lwork, int* info);
void dgesvd_(char* jobu, char* jobvt, int* m, int* n, double* a, int* lda, double* s, double* u, int* ldu, double* vt,
             int* ldvt, double* work, int* lwork, int* info)
{
    scipy_dgesvd_(jobu, jobvt, m, n, a, lda, s, u, ldu, vt, ldvt, work, lwork, info);
}
}
