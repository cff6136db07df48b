/* Oracle entry points (TEST INFRASTRUCTURE ONLY; see zeta64.c and ewald64.c). */
#ifndef ZETA64_H
#define ZETA64_H

#ifdef __cplusplus
extern "C" {
#endif

void z64_set_threads(int n);
int z64_tree(int n, const double* xyz, double box_r, const double* center, int max_depth, int* order,
             int* cell_depth, int* cell_body_off, int* cell_body_num, double* cell_center, int max_cells);
int z64_lists(int max_depth, int images, double cycle, double theta, long* n_p2p, long* n_m2l);
void z64_lists_fetch(int which, int* tgt, int* src, double* off);
int z64_solve(int n, const double* xyz, const double* q, double cycle, int P, int max_depth, int images,
              double theta, int stage_mask, double* pot, double* force, double* energy);
void z64_harmonics(int kind, int P, const double d[3], double* out);
void z64_apply(int kind, int P, const double d[3], const double* in, double* out);

int ew64_solve(int n, const double* xyz, const double* q, const double box[3], double eps, double rc,
               int n_tgt, const int* tgt, double* pot, double* force, int want_energy, double* energy);
/* Ewald energy and virial tensor Xi = -1/2 sum_pairs r_ij (x) F_ij (kJ/mol), 3 x 3 row-major. */
int ew64_virial(int n, const double* xyz, const double* q, const double box[3], double eps, double* energy,
                double* vir);
int direct64_solve(int n, const double* xyz, const double* q, double L, int nmax, double* pot, double* force);

#ifdef __cplusplus
}
#endif
#endif
