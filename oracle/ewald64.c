/*
 * ewald64 -- converged FP64 Ewald sum for orthorhombic periodic boxes (TEST INFRASTRUCTURE ONLY).
 *
 * This is the independent physics oracle: tin-foil (conducting) boundary, no
 * exclusions, neutralising background for a net charge.  It replaces the
 * reference's own Ewald (src/gromacs/rtfmm/ewald.cpp:11-238), whose parameters
 * (alpha = ksize/L with ksize 11, cutoff L/2, argument.cpp:19) truncate k-space
 * at about exp(-pi^2) ~ 5e-5 and so cannot serve as an FP64-grade reference.
 * The split is the standard one of that file: real space with erfc
 * (ewald.cpp:184-209), reciprocal space as a DFT over the atoms
 * (ewald.cpp:105-120, 212-238), and the self term (ewald.cpp:123-129).
 *
 * Accuracy control: alpha*rc = sqrt(-ln eps) + 0.3 and |k| cut where
 * exp(-k^2/(4 alpha^2)) < eps, so both truncation errors are ~eps relative.
 * Potentials and forces are evaluated for a subset of target atoms; the
 * structure factors always cover all atoms.
 * Units: positions nm, charges e; outputs in kJ/mol (ke = 138.935457833).
 */
#include "zeta64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KE_GMX 138.935457833

typedef struct { double re, im; } cplx;

static double wrap01(double x, double L)
{
    double y = fmod(x, L);
    if (y < 0) y += L;
    if (y >= L) y -= L;
    return y;
}

/* The Ewald sum; with 'vir' (and want_energy) also the virial tensor
 * Xi = -1/2 sum_pairs r_ij (x) F_ij = 1/2 dE/d(strain), row-major 3 x 3:
 * real space -1/4 sum_{i,j,n}' r_ijn (x) f_ijn, reciprocal space
 * 1/2 sum_k E_k [2 k k / k^2 (1 + k^2 / (4 alpha^2)) - I], the self and
 * background terms strain-free. */
static int ew64_core(int n, const double* xyz, const double* q, const double box[3], double eps, double rc_in,
                     int n_tgt, const int* tgt, double* pot, double* force, int want_energy, double* energy,
                     double* vir)
{
    if (n <= 0 || eps <= 0 || eps >= 1) return -1;
    double V = box[0] * box[1] * box[2];
    double Lmin = box[0];
    if (box[1] < Lmin) Lmin = box[1];
    if (box[2] < Lmin) Lmin = box[2];
    double s = sqrt(-log(eps)) + 0.3;
    double rc = rc_in;
    if (rc <= 0) {
        /* balance real space (targets x neighbours) against N x (#k) */
        int nt = want_energy ? n : n_tgt;
        double t = 1578.0 * V * V * (s * s * s * s * s * s) / (5.5 * 5.5 * 5.5 * 5.5 * 5.5 * 5.5) / (4.19 * (nt > 0 ? nt : 1));
        rc = pow(t, 1.0 / 6.0);
        if (rc < 0.8) rc = 0.8;
    }
    double alpha = s / rc;
    /* k cut: exp(-k^2/4a^2) = eps  =>  k = 2 a s */
    double kcut = 2.0 * alpha * s;
    int kmx[3];
    for (int d = 0; d < 3; d++) kmx[d] = (int)ceil(kcut * box[d] / (2 * M_PI));

    /* half space of k vectors: (kx>0) or (kx==0 && ky>0) or (kx==0 && ky==0 && kz>0) */
    int nkcap = (kmx[0] + 1) * (2 * kmx[1] + 1) * (2 * kmx[2] + 1);
    int* kv = (int*)malloc(sizeof(int) * 3 * nkcap);
    double* kw = (double*)malloc(sizeof(double) * nkcap);
    int nk = 0;
    for (int a = 0; a <= kmx[0]; a++)
        for (int b = -kmx[1]; b <= kmx[1]; b++)
            for (int c = -kmx[2]; c <= kmx[2]; c++) {
                if (a == 0 && (b < 0 || (b == 0 && c <= 0))) continue;
                double kx = 2 * M_PI * a / box[0], ky = 2 * M_PI * b / box[1], kz = 2 * M_PI * c / box[2];
                double k2 = kx * kx + ky * ky + kz * kz;
                if (k2 > kcut * kcut) continue;
                kv[3 * nk] = a; kv[3 * nk + 1] = b; kv[3 * nk + 2] = c;
                /* factor 2 for the -k partner */
                kw[nk] = 2.0 * (4 * M_PI / V) * exp(-k2 / (4 * alpha * alpha)) / k2;
                nk++;
            }

    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    int K0 = kmx[0] + 1, K1 = 2 * kmx[1] + 1, K2 = 2 * kmx[2] + 1;
    /* structure factors S(k) = sum_j q_j exp(i k.r_j) */
    cplx* S = (cplx*)calloc(nk, sizeof(cplx));
    cplx* Sth = (cplx*)calloc((size_t)nk * nth, sizeof(cplx));
#pragma omp parallel
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        cplx* Sl = Sth + (size_t)tid * nk;
        cplx* ex = (cplx*)malloc(sizeof(cplx) * K0);
        cplx* ey = (cplx*)malloc(sizeof(cplx) * K1);
        cplx* ez = (cplx*)malloc(sizeof(cplx) * K2);
#pragma omp for schedule(static)
        for (int j = 0; j < n; j++) {
            double th[3];
            for (int d = 0; d < 3; d++) th[d] = 2 * M_PI * xyz[3 * j + d] / box[d];
            for (int a = 0; a < K0; a++) { ex[a].re = cos(a * th[0]); ex[a].im = sin(a * th[0]); }
            for (int b = -kmx[1]; b <= kmx[1]; b++) { ey[b + kmx[1]].re = cos(b * th[1]); ey[b + kmx[1]].im = sin(b * th[1]); }
            for (int c = -kmx[2]; c <= kmx[2]; c++) { ez[c + kmx[2]].re = cos(c * th[2]); ez[c + kmx[2]].im = sin(c * th[2]); }
            for (int k = 0; k < nk; k++) {
                cplx A = ex[kv[3 * k]], B = ey[kv[3 * k + 1] + kmx[1]], C = ez[kv[3 * k + 2] + kmx[2]];
                double abr = A.re * B.re - A.im * B.im, abi = A.re * B.im + A.im * B.re;
                Sl[k].re += q[j] * (abr * C.re - abi * C.im);
                Sl[k].im += q[j] * (abr * C.im + abi * C.re);
            }
        }
        free(ex); free(ey); free(ez);
    }
    for (int t = 0; t < nth; t++)
        for (int k = 0; k < nk; k++) { S[k].re += Sth[(size_t)t * nk + k].re; S[k].im += Sth[(size_t)t * nk + k].im; }
    free(Sth);

    double Q = 0;
    for (int j = 0; j < n; j++) Q += q[j];

    /* cell list for real space */
    int g[3];
    double cw[3];
    int R[3];
    for (int d = 0; d < 3; d++) {
        g[d] = (int)floor(box[d] / (rc / 2));
        if (g[d] < 1) g[d] = 1;
        cw[d] = box[d] / g[d];
        R[d] = (int)ceil(rc / cw[d]);
    }
    int ncell = g[0] * g[1] * g[2];
    int* head = (int*)malloc(sizeof(int) * (ncell + 1));
    int* lst = (int*)malloc(sizeof(int) * n);
    double* wx = (double*)malloc(sizeof(double) * 3 * n);
    {
        int* cnt = (int*)calloc(ncell + 1, sizeof(int));
        int* cid = (int*)malloc(sizeof(int) * n);
        for (int j = 0; j < n; j++) {
            int ci[3];
            for (int d = 0; d < 3; d++) {
                wx[3 * j + d] = wrap01(xyz[3 * j + d], box[d]);
                ci[d] = (int)(wx[3 * j + d] / cw[d]);
                if (ci[d] >= g[d]) ci[d] = g[d] - 1;
            }
            cid[j] = (ci[0] * g[1] + ci[1]) * g[2] + ci[2];
            cnt[cid[j] + 1]++;
        }
        for (int c = 0; c < ncell; c++) cnt[c + 1] += cnt[c];
        memcpy(head, cnt, sizeof(int) * (ncell + 1));
        for (int j = 0; j < n; j++) lst[cnt[cid[j]]++] = j;
        free(cnt); free(cid);
    }

    int ntg = want_energy ? n : n_tgt;
    double* epart = (double*)calloc(ntg > 0 ? ntg : 1, sizeof(double));
    double* vpart = vir ? (double*)calloc(6 * (size_t)(ntg > 0 ? ntg : 1), sizeof(double)) : NULL;
    const double rc2 = rc * rc;
    const double tsp = 2.0 / sqrt(M_PI);
#pragma omp parallel
    {
        cplx* ex = (cplx*)malloc(sizeof(cplx) * K0);
        cplx* ey = (cplx*)malloc(sizeof(cplx) * K1);
        cplx* ez = (cplx*)malloc(sizeof(cplx) * K2);
#pragma omp for schedule(dynamic, 8)
        for (int t = 0; t < ntg; t++) {
            int i = want_energy ? t : tgt[t];
            double xi[3] = {wx[3 * i], wx[3 * i + 1], wx[3 * i + 2]};
            int ci[3];
            for (int d = 0; d < 3; d++) {
                ci[d] = (int)(xi[d] / cw[d]);
                if (ci[d] >= g[d]) ci[d] = g[d] - 1;
            }
            double phi = 0, f[3] = {0, 0, 0};
            double w6[6] = {0, 0, 0, 0, 0, 0};  /* sum_j fs d (x) d (xx, yy, zz, xy, xz, yz) */
            for (int ox = -R[0]; ox <= R[0]; ox++) {
                int cx = ci[0] + ox;
                int wxi = ((cx % g[0]) + g[0]) % g[0];
                double sx = (double)((cx - wxi) / g[0]) * box[0];
                for (int oy = -R[1]; oy <= R[1]; oy++) {
                    int cy = ci[1] + oy;
                    int wyi = ((cy % g[1]) + g[1]) % g[1];
                    double sy = (double)((cy - wyi) / g[1]) * box[1];
                    for (int oz = -R[2]; oz <= R[2]; oz++) {
                        int cz = ci[2] + oz;
                        int wzi = ((cz % g[2]) + g[2]) % g[2];
                        double sz = (double)((cz - wzi) / g[2]) * box[2];
                        int c = (wxi * g[1] + wyi) * g[2] + wzi;
                        for (int p = head[c]; p < head[c + 1]; p++) {
                            int j = lst[p];
                            double d0 = xi[0] - (wx[3 * j] + sx);
                            double d1 = xi[1] - (wx[3 * j + 1] + sy);
                            double d2 = xi[2] - (wx[3 * j + 2] + sz);
                            double r2 = d0 * d0 + d1 * d1 + d2 * d2;
                            if (r2 >= rc2 || r2 == 0) continue;
                            double r = sqrt(r2);
                            double ec = erfc(alpha * r);
                            phi += q[j] * ec / r;
                            double fs = q[j] * (ec / r + tsp * alpha * exp(-alpha * alpha * r2)) / r2;
                            f[0] += fs * d0; f[1] += fs * d1; f[2] += fs * d2;
                            if (vir) {
                                w6[0] += fs * d0 * d0; w6[1] += fs * d1 * d1; w6[2] += fs * d2 * d2;
                                w6[3] += fs * d0 * d1; w6[4] += fs * d0 * d2; w6[5] += fs * d1 * d2;
                            }
                        }
                    }
                }
            }
            /* reciprocal space */
            double th[3];
            for (int d = 0; d < 3; d++) th[d] = 2 * M_PI * xyz[3 * i + d] / box[d];
            for (int a = 0; a < K0; a++) { ex[a].re = cos(a * th[0]); ex[a].im = sin(a * th[0]); }
            for (int b = -kmx[1]; b <= kmx[1]; b++) { ey[b + kmx[1]].re = cos(b * th[1]); ey[b + kmx[1]].im = sin(b * th[1]); }
            for (int c = -kmx[2]; c <= kmx[2]; c++) { ez[c + kmx[2]].re = cos(c * th[2]); ez[c + kmx[2]].im = sin(c * th[2]); }
            for (int k = 0; k < nk; k++) {
                cplx A = ex[kv[3 * k]], B = ey[kv[3 * k + 1] + kmx[1]], C = ez[kv[3 * k + 2] + kmx[2]];
                double abr = A.re * B.re - A.im * B.im, abi = A.re * B.im + A.im * B.re;
                double er = abr * C.re - abi * C.im, ei = abr * C.im + abi * C.re; /* exp(i k.r_i) */
                /* Re[S conj(e)] = sum_j q_j cos(k.(r_j - r_i)) */
                double re = S[k].re * er + S[k].im * ei;
                double im = S[k].im * er - S[k].re * ei; /* sum_j q_j sin(k.(r_j - r_i)) */
                phi += kw[k] * re;
                double kx = 2 * M_PI * kv[3 * k] / box[0], ky = 2 * M_PI * kv[3 * k + 1] / box[1],
                       kz = 2 * M_PI * kv[3 * k + 2] / box[2];
                /* E_i = -grad_i phi = -kw * sum_j q_j sin(k.(r_j - r_i)) * k */
                f[0] -= kw[k] * im * kx;
                f[1] -= kw[k] * im * ky;
                f[2] -= kw[k] * im * kz;
            }
            /* self and neutralising background */
            phi -= tsp * alpha * q[i];
            phi -= M_PI * Q / (V * alpha * alpha);
            if (want_energy) epart[t] = q[i] * phi;
            if (vir && want_energy)
                for (int c = 0; c < 6; c++) vpart[6 * (size_t)t + c] = q[i] * w6[c];
            if (pot) pot[t] = phi * KE_GMX;
            if (force) {
                force[3 * t] = q[i] * f[0] * KE_GMX;
                force[3 * t + 1] = q[i] * f[1] * KE_GMX;
                force[3 * t + 2] = q[i] * f[2] * KE_GMX;
            }
        }
        free(ex); free(ey); free(ez);
    }
    if (want_energy && energy) {
        double e = 0;
        for (int t = 0; t < ntg; t++) e += epart[t];
        *energy = 0.5 * e * KE_GMX;
    }
    if (vir && want_energy) {
        double w6[6] = {0, 0, 0, 0, 0, 0};
        for (int t = 0; t < ntg; t++)
            for (int c = 0; c < 6; c++) w6[c] += vpart[6 * (size_t)t + c];
        /* reciprocal space: E_k = 1/2 kw |S_k|^2 per half-space vector */
        double r6[6] = {0, 0, 0, 0, 0, 0};
        for (int k = 0; k < nk; k++) {
            double kx = 2 * M_PI * kv[3 * k] / box[0], ky = 2 * M_PI * kv[3 * k + 1] / box[1],
                   kz = 2 * M_PI * kv[3 * k + 2] / box[2];
            double k2 = kx * kx + ky * ky + kz * kz;
            double Ek = 0.5 * kw[k] * (S[k].re * S[k].re + S[k].im * S[k].im);
            double b = 2.0 * (1.0 + k2 / (4 * alpha * alpha)) / k2;
            r6[0] += Ek * (b * kx * kx - 1); r6[1] += Ek * (b * ky * ky - 1); r6[2] += Ek * (b * kz * kz - 1);
            r6[3] += Ek * b * kx * ky; r6[4] += Ek * b * kx * kz; r6[5] += Ek * b * ky * kz;
        }
        double v6[6];
        for (int c = 0; c < 6; c++) v6[c] = (-0.25 * w6[c] + 0.5 * r6[c]) * KE_GMX;
        vir[0] = v6[0]; vir[4] = v6[1]; vir[8] = v6[2];
        vir[1] = vir[3] = v6[3];
        vir[2] = vir[6] = v6[4];
        vir[5] = vir[7] = v6[5];
    }
    free(vpart);
    free(epart); free(head); free(lst); free(wx); free(S); free(kv); free(kw);
    return nk;
}

int ew64_solve(int n, const double* xyz, const double* q, const double box[3], double eps, double rc_in,
               int n_tgt, const int* tgt, double* pot, double* force, int want_energy, double* energy)
{
    return ew64_core(n, xyz, q, box, eps, rc_in, n_tgt, tgt, pot, force, want_energy, energy, NULL);
}

int ew64_virial(int n, const double* xyz, const double* q, const double box[3], double eps, double* energy,
                double* vir)
{
    return ew64_core(n, xyz, q, box, eps, 0.0, 0, NULL, NULL, NULL, 1, energy, vir);
}

/* Direct lattice sum in spherical shells for tiny systems, tin-foil corrected:
 * phi_i = sum_{|n|<=nmax}' q_j/|r_i - r_j - nL| over shells, then the surface term
 * (4 pi / 3V) M.r_i is removed.  Used only to check ew64_solve on a few atoms. */
int direct64_solve(int n, const double* xyz, const double* q, double L, int nmax, double* pot, double* force)
{
    double V = L * L * L;
    double M[3] = {0, 0, 0};
    for (int j = 0; j < n; j++)
        for (int d = 0; d < 3; d++) M[d] += q[j] * xyz[3 * j + d];
    double c = 4 * M_PI / (3 * V);
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; i++) {
        double phi = 0, f[3] = {0, 0, 0};
        for (int a = -nmax; a <= nmax; a++)
            for (int b = -nmax; b <= nmax; b++)
                for (int e = -nmax; e <= nmax; e++) {
                    if (a * a + b * b + e * e > nmax * nmax) continue;
                    for (int j = 0; j < n; j++) {
                        double d0 = xyz[3 * i] - xyz[3 * j] - a * L;
                        double d1 = xyz[3 * i + 1] - xyz[3 * j + 1] - b * L;
                        double d2 = xyz[3 * i + 2] - xyz[3 * j + 2] - e * L;
                        double r2 = d0 * d0 + d1 * d1 + d2 * d2;
                        if (r2 == 0) continue;
                        double r = sqrt(r2);
                        phi += q[j] / r;
                        double s = q[j] / (r2 * r);
                        f[0] += s * d0; f[1] += s * d1; f[2] += s * d2;
                    }
                }
        /* spherical summation equals tin-foil plus the surface term; remove it */
        phi -= c * (M[0] * xyz[3 * i] + M[1] * xyz[3 * i + 1] + M[2] * xyz[3 * i + 2]);
        for (int d = 0; d < 3; d++) f[d] += c * M[d];
        pot[i] = phi * KE_GMX;
        for (int d = 0; d < 3; d++) force[3 * i + d] = q[i] * f[d] * KE_GMX;
    }
    return 0;
}
