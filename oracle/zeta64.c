/*
 * zeta64 -- FP64 CPU restatement of the zeta_fmm GPU FMM (TEST INFRASTRUCTURE ONLY).
 *
 * This file is the parity oracle.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load it; the product library never does.
 *
 * Every routine restates, in plain C and double precision, the reference
 * algorithm of jooooow/GROMACS-FMM, src/gromacs/zeta_fmm/:
 *   - solid harmonics          kernel.cu:98-217   (calc_Ynm, calc_YnmD, calc_Ynm2)
 *   - P2M                      kernel.cu:219-242
 *   - M2M / image M2M          kernel.cu:310-406
 *   - L2L                      kernel.cu:408-454
 *   - P2P                      kernel.cu:456-496
 *   - M2L (j+n<=P truncation)  kernel.cu:550-606
 *   - L2P                      kernel.cu:608-656 (+ derivate_sph2cart :80-96)
 *   - launch order             kernel.cu:815-896 (P2M, M2M, image M2M, M2L, P2P, L2L, L2P)
 *   - tree                     tree.cpp:13-99    (BFS complete octree, counting sort by octant)
 *   - traversal                traverser.cpp:9-214 (MAC, dual-tree recursion, periodic near/far)
 *   - unit conversion          gpu_solver.cu:250-256
 *   - dipole correction        solver.cpp:30-49
 *   - sort back to input order solver.cpp:51-67
 *   - energy 0.5*sum(q*phi)    fmm.cpp:89-98
 * Per-cell loops are OpenMP-parallel where the reference's kernels are
 * parallel over cells (each cell writes only its own expansion or bodies).
 *
 * Pinning: the tree and lists equal fixtures made by the reference's own
 * tree.cpp/traverser.cpp bit for bit, and the potentials and forces (before the
 * dipole correction) equal those of the reference's own FP64 kernels, run on the
 * host by oracle/ref_kernels_driver.cpp, to 1e-12 relative (5e-16 measured) on
 * the configurations of tests/golden/ref_outputs.npz.
 */
#include "zeta64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KE_GMX 138.935457833  /* gmx::c_one4PiEps0, kJ mol^-1 nm e^-2 (units.h:110) */

typedef struct { double re, im; } zc;

static inline zc zc_make(double r, double i) { zc c; c.re = r; c.im = i; return c; }
static inline zc zc_mul(zc a, zc b) { return zc_make(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline zc zc_scale(zc a, double s) { return zc_make(a.re * s, a.im * s); }
static inline zc zc_conj(zc a) { return zc_make(a.re, -a.im); }
static inline void zc_acc(zc* a, zc b) { a->re += b.re; a->im += b.im; }
static inline int neg1pow(int n) { return (n & 1) ? -1 : 1; }         /* oddOrEven, kernel.cu:69 */
static inline int ipow2n(int m) { return m >= 0 ? 1 : neg1pow(m); }    /* kernel.cu:74 */
static inline int npack(int P) { return (P + 1) * (P + 2) / 2; }        /* type.h:30 */

/* vec3r::toSph2 (type.h:376-385): clamped acos, atan2. */
static void to_sph(const double d[3], double* rho, double* th, double* ph)
{
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double c = d[2] / r;
    if (c < -1) c = -1;
    else if (c > 1) c = 1;
    *rho = r;
    *th = (r == 0) ? 0 : acos(c);
    *ph = atan2(d[1], d[0]);
}

/* Regular solid harmonics, index n*n+n+m, m in [-n,n] (kernel.cu:98-138). */
static void harm_regular(zc* Y, int P, double rho, double th, double ph)
{
    double x = cos(th), y = sin(th);
    double fact = 1, pn = 1, rhom = 1;
    zc ei = zc_make(cos(ph), sin(ph));
    zc eim = zc_make(1, 0);
    for (int m = 0; m <= P; m++) {
        double p = pn;
        Y[m * m + 2 * m] = zc_scale(eim, rhom * p);
        Y[m * m] = zc_conj(Y[m * m + 2 * m]);
        double p1 = p;
        p = x * (2 * m + 1) * p1;
        rhom *= rho;
        double rhon = rhom;
        for (int n = m + 1; n <= P; n++) {
            rhon /= -(n + m);
            Y[n * n + n + m] = zc_scale(eim, rhon * p);
            Y[n * n + n - m] = zc_conj(Y[n * n + n + m]);
            double p2 = p1;
            p1 = p;
            p = (x * (2 * n + 1) * p1 - (n + m) * p2) / (n - m + 1);
            rhon *= rho;
        }
        rhom /= -(2 * m + 2) * (2 * m + 1);
        pn = -pn * fact * y;
        fact += 2;
        eim = zc_mul(eim, ei);
    }
}

/* Theta-derivative of the regular harmonics, m >= 0 entries only (kernel.cu:140-177). */
static void harm_regular_dtheta(zc* YD, int P, double rho, double th, double ph)
{
    double x = cos(th), y = sin(th);
    double invy = (y == 0) ? 0 : 1 / y;
    double fact = 1, pn = 1, rhom = 1;
    zc ei = zc_make(cos(ph), sin(ph));
    zc eim = zc_make(1, 0);
    for (int m = 0; m <= P; m++) {
        double p = pn;
        double p1 = p;
        p = x * (2 * m + 1) * p1;
        YD[m * m + 2 * m] = zc_scale(eim, rhom * (p - (m + 1) * x * p1) * invy);
        rhom *= rho;
        double rhon = rhom;
        for (int n = m + 1; n <= P; n++) {
            rhon /= -(n + m);
            double p2 = p1;
            p1 = p;
            p = (x * (2 * n + 1) * p1 - (n + m) * p2) / (n - m + 1);
            YD[n * n + n + m] = zc_scale(eim, rhon * ((n - m + 1) * p - (n + 1) * x * p1) * invy);
            rhon *= rho;
        }
        rhom /= -(2 * m + 2) * (2 * m + 1);
        pn = -pn * fact * y;
        fact += 2;
        eim = zc_mul(eim, ei);
    }
}

/* Singular solid harmonics (kernel.cu:179-217). */
static void harm_singular(zc* Y, int P, double rho, double th, double ph)
{
    double x = cos(th), y = sin(th);
    double fact = 1, pn = 1;
    double inv_r = -1.0 / rho;
    double rhom = -inv_r;
    zc ei = zc_make(cos(ph), sin(ph));
    zc eim = zc_make(1, 0);
    for (int m = 0; m <= P; m++) {
        double p = pn;
        Y[m * m + 2 * m] = zc_scale(eim, rhom * p);
        Y[m * m] = zc_conj(Y[m * m + 2 * m]);
        double p1 = p;
        p = x * (2 * m + 1) * p1;
        rhom *= inv_r;
        double rhon = rhom;
        for (int n = m + 1; n <= P; n++) {
            Y[n * n + n + m] = zc_scale(eim, rhon * p);
            Y[n * n + n - m] = zc_conj(Y[n * n + n + m]);
            double p2 = p1;
            p1 = p;
            p = (x * (2 * n + 1) * p1 - (n + m) * p2) / (n - m + 1);
            rhon *= inv_r * (n - m + 1);
        }
        pn = -pn * fact * y;
        fact += 2;
        eim = zc_mul(eim, ei);
    }
}

/* ---------------------------------------------------------------- operators */

/* P2M for one body into packed M (kernel.cu:228-240; harmonics taken at -phi). */
static void op_p2m(int P, zc* Ywork, const double dx[3], double q, zc* M)
{
    double rho, th, ph;
    to_sph(dx, &rho, &th, &ph);
    harm_regular(Ywork, P, rho, th, -ph);
    for (int n = 0; n <= P; n++)
        for (int m = 0; m <= n; m++)
            zc_acc(&M[n * (n + 1) / 2 + m], zc_scale(Ywork[n * n + n + m], q));
}

/* Child M -> parent M with dx = parent centre - child centre (kernel.cu:325-351). */
static void op_m2m(int P, zc* Y, const double dx[3], const zc* Mc, zc* Mp)
{
    double rho, th, ph;
    to_sph(dx, &rho, &th, &ph);
    harm_regular(Y, P, rho, th, ph);
    for (int j = 0; j <= P; j++) {
        for (int k = 0; k <= j; k++) {
            zc acc = zc_make(0, 0);
            for (int n = 0; n <= j; n++) {
                int lo = (-n > -j + k + n) ? -n : (-j + k + n);
                int hi = (k - 1 < n) ? (k - 1) : n;
                for (int m = lo; m <= hi; m++) {
                    zc t = zc_mul(Mc[(j - n) * (j - n + 1) / 2 + k - m], Y[n * n + n - m]);
                    zc_acc(&acc, zc_scale(t, (double)(ipow2n(m) * neg1pow(n))));
                }
                int hi2 = (n < j + k - n) ? n : (j + k - n);
                for (int m = k; m <= hi2; m++) {
                    zc t = zc_mul(zc_conj(Mc[(j - n) * (j - n + 1) / 2 - k + m]), Y[n * n + n - m]);
                    zc_acc(&acc, zc_scale(t, (double)neg1pow(k + n + m)));
                }
            }
            zc_acc(&Mp[j * (j + 1) / 2 + k], acc);
        }
    }
}

/* Parent L -> child L with dX = child centre - parent centre (kernel.cu:422-451). */
static void op_l2l(int P, zc* Y, const double dX[3], const zc* Lp, zc* Lc)
{
    double rho, th, ph;
    to_sph(dX, &rho, &th, &ph);
    harm_regular(Y, P, rho, th, ph);
    for (int j = 0; j <= P; j++) {
        for (int k = 0; k <= j; k++) {
            zc acc = zc_make(0, 0);
            for (int n = j; n <= P; n++) {
                for (int m = j + k - n; m < 0; m++) {
                    int jnkm = (n - j) * (n - j) + n - j + m - k;
                    zc t = zc_mul(zc_conj(Lp[n * (n + 1) / 2 - m]), Y[jnkm]);
                    zc_acc(&acc, zc_scale(t, (double)neg1pow(k)));
                }
                for (int m = 0; m <= n; m++) {
                    if (n - j >= abs(m - k)) {
                        int jnkm = (n - j) * (n - j) + n - j + m - k;
                        zc t = zc_mul(Lp[n * (n + 1) / 2 + m], Y[jnkm]);
                        zc_acc(&acc, zc_scale(t, (double)neg1pow((m - k) * (m < k))));
                    }
                }
            }
            zc_acc(&Lc[j * (j + 1) / 2 + k], acc);
        }
    }
}

/* Source M -> target L with dX = target centre - (source centre + offset) (kernel.cu:572-603). */
static void op_m2l(int P, zc* Y, const double dX[3], const zc* Ms, zc* Lt)
{
    double rho, th, ph;
    to_sph(dX, &rho, &th, &ph);
    harm_singular(Y, P, rho, th, ph);
    for (int j = 0; j <= P; j++) {
        double cnm = neg1pow(j);
        for (int k = 0; k <= j; k++) {
            zc acc = zc_make(0, 0);
            for (int n = 0; n + j <= P; n++) {
                for (int m = -n; m < 0; m++) {
                    int jnkm = (j + n) * (j + n) + j + n + m - k;
                    zc t = zc_mul(zc_conj(Ms[n * (n + 1) / 2 - m]), Y[jnkm]);
                    zc_acc(&acc, zc_scale(t, cnm));
                }
                for (int m = 0; m <= n; m++) {
                    int jnkm = (j + n) * (j + n) + j + n + m - k;
                    double c2 = cnm * neg1pow((k - m) * (k < m) + m);
                    zc t = zc_mul(Ms[n * (n + 1) / 2 + m], Y[jnkm]);
                    zc_acc(&acc, zc_scale(t, c2));
                }
            }
            zc_acc(&Lt[j * (j + 1) / 2 + k], acc);
        }
    }
}

/* derivate_sph2cart (kernel.cu:80-96). */
static void sph_grad_to_cart(double rho, double th, double ph, const double g[3], double out[3])
{
    double st = sin(th);
    double ist = (st == 0) ? 0 : 1 / st;
    double ir = (rho == 0) ? 0 : 1 / rho;
    out[0] = st * cos(ph) * g[0] + cos(th) * cos(ph) * ir * g[1] - sin(ph) * ir * ist * g[2];
    out[1] = st * sin(ph) * g[0] + cos(th) * sin(ph) * ir * g[1] + cos(ph) * ir * ist * g[2];
    out[2] = cos(th) * g[0] - st * ir * g[1];
}

/* L2P for one body: potential and gradient (kernel.cu:624-654). */
static void op_l2p(int P, zc* Y, zc* YD, const double dx[3], const zc* L, double* pot, double grad[3])
{
    double rho, th, ph;
    to_sph(dx, &rho, &th, &ph);
    harm_regular(Y, P, rho, th, ph);
    harm_regular_dtheta(YD, P, rho, th, ph);
    double p = 0, t[3] = {0, 0, 0};
    for (int n = 0; n <= P; n++) {
        int nm = n * n + n, nms = n * (n + 1) / 2;
        zc ly = zc_mul(L[nms], Y[nm]);
        p += ly.re;
        t[0] += ly.re / rho * n;
        t[1] += zc_mul(L[nms], YD[nm]).re;
        for (int m = 1; m <= n; m++) {
            nm = n * n + n + m;
            nms = n * (n + 1) / 2 + m;
            ly = zc_mul(L[nms], Y[nm]);
            p += 2 * ly.re;
            t[0] += 2 * ly.re / rho * n;
            t[1] += 2 * zc_mul(L[nms], YD[nm]).re;
            t[2] += 2 * zc_mul(ly, zc_make(0, 1)).re * m;
        }
    }
    double c[3];
    sph_grad_to_cart(rho, th, ph, t, c);
    *pot += p;
    grad[0] += c[0];
    grad[1] += c[1];
    grad[2] += c[2];
}

/* ---------------------------------------------------------------- tree */

typedef struct {
    int depth;
    double r;
    double c[3];
    int child_off, child_num;
    int body_off, body_num;
} zcell;

typedef struct {
    int ncell, cap;
    zcell* v;
} zcells;

static void cells_push(zcells* cs, zcell c)
{
    if (cs->ncell == cs->cap) {
        cs->cap = cs->cap ? 2 * cs->cap : 64;
        cs->v = (zcell*)realloc(cs->v, sizeof(zcell) * cs->cap);
    }
    cs->v[cs->ncell++] = c;
}

static inline int octant_of(const double* x, const double* c)
{
    return ((x[0] > c[0]) << 2) + ((x[1] > c[1]) << 1) + ((x[2] > c[2]) << 0);
}

/* CompleteBalancedOctree::build (tree.cpp:13-99).  order[i] = input index of the
 * body at sorted position i; bodies are permuted in place through 'order'. */
static void build_tree(int n, const double* xyz, double box_r, const double* center, int max_depth,
                       zcells* cs, int* order)
{
    for (int i = 0; i < n; i++) order[i] = i;
    int* buf = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    zcell root;
    root.depth = 0;
    root.r = box_r;
    root.c[0] = center[0]; root.c[1] = center[1]; root.c[2] = center[2];
    root.child_off = 0; root.child_num = 0;
    root.body_off = 0; root.body_num = n;
    cells_push(cs, root);
    /* BFS queue == cell index order, since every split appends 8 children. */
    for (int head = 0; head < cs->ncell; head++) {
        zcell bc = cs->v[head];
        if (bc.depth >= max_depth) continue;
        int begin = bc.body_off, num = bc.body_num;
        int cnt[8] = {0}, off[8];
        for (int i = begin; i < begin + num; i++) cnt[octant_of(&xyz[3 * order[i]], bc.c)]++;
        int s = 0;
        for (int o = 0; o < 8; o++) { off[o] = s; s += cnt[o]; }
        for (int i = begin; i < begin + num; i++) {
            int o = octant_of(&xyz[3 * order[i]], bc.c);
            buf[off[o]++] = order[i];
        }
        for (int i = 0; i < num; i++) order[begin + i] = buf[i];
        int ins = cs->ncell;
        cs->v[head].child_off = ins;
        cs->v[head].child_num = 8;
        double h = bc.r / 2;
        for (int o = 0; o < 8; o++) {
            zcell ch;
            ch.depth = bc.depth + 1;
            ch.r = bc.r / 2;
            ch.child_off = 0; ch.child_num = 0;
            ch.body_off = begin + off[o] - cnt[o];
            ch.body_num = cnt[o];
            ch.c[0] = bc.c[0] + ((o & 4) ? h : -h);
            ch.c[1] = bc.c[1] + ((o & 2) ? h : -h);
            ch.c[2] = bc.c[2] + ((o & 1) ? h : -h);
            cells_push(cs, ch);
        }
    }
    free(buf);
}

/* ---------------------------------------------------------------- traversal */

typedef struct {
    long n, cap;
    int* tgt;
    int* src;
    double* off; /* 3 per entry */
} zlist;

static void list_push(zlist* l, int t, int s, const double o[3])
{
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 1024;
        l->tgt = (int*)realloc(l->tgt, sizeof(int) * l->cap);
        l->src = (int*)realloc(l->src, sizeof(int) * l->cap);
        l->off = (double*)realloc(l->off, sizeof(double) * 3 * l->cap);
    }
    l->tgt[l->n] = t;
    l->src[l->n] = s;
    l->off[3 * l->n + 0] = o[0];
    l->off[3 * l->n + 1] = o[1];
    l->off[3 * l->n + 2] = o[2];
    l->n++;
}

typedef struct {
    const zcells* cs;
    double theta;
    zlist p2p, m2l;
} ztrav;

/* NearFieldSelector::is_near with MAC (traverser.cpp:9-22). */
static int is_near(const zcell* a, const zcell* b, const double off[3], double theta)
{
    double d0 = a->c[0] - b->c[0] - off[0];
    double d1 = a->c[1] - b->c[1] - off[1];
    double d2 = a->c[2] - b->c[2] - off[2];
    double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2) * theta;
    return !(r > a->r + b->r);
}

/* Traverser::horizontal (traverser.cpp:88-141). */
static void horizontal(ztrav* t, int a, int b, const double off[3])
{
    const zcell* A = &t->cs->v[a];
    const zcell* B = &t->cs->v[b];
    if (!is_near(A, B, off, t->theta)) {
        list_push(&t->m2l, a, b, off);
        return;
    }
    if (A->child_num == 0 && B->child_num == 0) {
        list_push(&t->p2p, a, b, off);
    } else if (A->child_num == 0) {
        for (int i = 0; i < B->child_num; i++) horizontal(t, a, B->child_off + i, off);
    } else if (B->child_num == 0) {
        for (int i = 0; i < A->child_num; i++) horizontal(t, A->child_off + i, b, off);
    } else if (A->r >= B->r) {
        for (int i = 0; i < A->child_num; i++) horizontal(t, A->child_off + i, b, off);
    } else {
        for (int i = 0; i < B->child_num; i++) horizontal(t, a, B->child_off + i, off);
    }
}

static int cmp_long_pair(const void* pa, const void* pb)
{
    const long* a = (const long*)pa;
    const long* b = (const long*)pb;
    if (a[0] != b[0]) return a[0] < b[0] ? -1 : 1;
    if (a[1] != b[1]) return a[1] < b[1] ? -1 : 1;
    return 0;
}

/* std::map<int, vector> iteration order: ascending target, append order within. */
static void list_group_by_target(zlist* l)
{
    long n = l->n;
    if (n == 0) return;
    long* key = (long*)malloc(sizeof(long) * 2 * n);
    for (long i = 0; i < n; i++) { key[2 * i] = l->tgt[i]; key[2 * i + 1] = i; }
    qsort(key, n, 2 * sizeof(long), cmp_long_pair);
    int* t2 = (int*)malloc(sizeof(int) * n);
    int* s2 = (int*)malloc(sizeof(int) * n);
    double* o2 = (double*)malloc(sizeof(double) * 3 * n);
    for (long i = 0; i < n; i++) {
        long j = key[2 * i + 1];
        t2[i] = l->tgt[j];
        s2[i] = l->src[j];
        o2[3 * i] = l->off[3 * j]; o2[3 * i + 1] = l->off[3 * j + 1]; o2[3 * i + 2] = l->off[3 * j + 2];
    }
    free(l->tgt); free(l->src); free(l->off); free(key);
    l->tgt = t2; l->src = s2; l->off = o2;
}

/* Traverser::traverse (traverser.cpp:47-67) with periodic near (:143-160) and far (:162-214).
 * Image cells are appended to 'cs' (depth -1-m, child = previous image or root). */
static void traverse(zcells* cs, double theta, int images, double cycle, ztrav* t, int* n_img_out)
{
    memset(t, 0, sizeof(*t));
    t->theta = theta;
    t->cs = cs;
    double zero[3] = {0, 0, 0};
    int nimg = 0;
    if (images == 0) {
        horizontal(t, 0, 0, zero);
    } else {
        for (int pz = -1; pz <= 1; pz++)
            for (int py = -1; py <= 1; py++)
                for (int px = -1; px <= 1; px++) {
                    double o[3] = {px * cycle, py * cycle, pz * cycle};
                    horizontal(t, 0, 0, o);
                }
        int first = cs->ncell, child = 0;
        for (int m = 0; m < images - 1; m++) {
            zcell c;
            memset(&c, 0, sizeof(c));
            c.depth = -1 - m;
            c.c[0] = cs->v[child].c[0]; c.c[1] = cs->v[child].c[1]; c.c[2] = cs->v[child].c[2];
            c.child_off = child;
            c.child_num = 1;
            cells_push(cs, c);
            t->cs = cs;
            child = cs->ncell - 1;
            nimg++;
        }
        double cyc = cycle;
        int idx = first;
        for (int m = 0; m < images - 1; m++) {
            for (int pz = -1; pz <= 1; pz++)
                for (int py = -1; py <= 1; py++)
                    for (int px = -1; px <= 1; px++) {
                        if (px == 0 && py == 0 && pz == 0) continue;
                        for (int cz = -1; cz <= 1; cz++)
                            for (int cy = -1; cy <= 1; cy++)
                                for (int cx = -1; cx <= 1; cx++) {
                                    double o[3] = {(px * 3 + cx) * cyc, (py * 3 + cy) * cyc, (pz * 3 + cz) * cyc};
                                    list_push(&t->m2l, 0, cs->v[idx].child_off, o);
                                }
                    }
            idx++;
            cyc *= 3;
        }
    }
    list_group_by_target(&t->p2p);
    list_group_by_target(&t->m2l);
    *n_img_out = nimg;
}

/* ---------------------------------------------------------------- C API */

static int g_nthreads = 0;

void z64_set_threads(int n) { g_nthreads = n; }

static void set_omp(void)
{
#ifdef _OPENMP
    if (g_nthreads > 0) omp_set_num_threads(g_nthreads);
#endif
}

int z64_tree(int n, const double* xyz, double box_r, const double* center, int max_depth,
             int* order, int* cell_depth, int* cell_body_off, int* cell_body_num, double* cell_center,
             int max_cells)
{
    zcells cs = {0, 0, NULL};
    build_tree(n, xyz, box_r, center, max_depth, &cs, order);
    int nc = cs.ncell;
    if (nc > max_cells) { free(cs.v); return -1; }
    for (int i = 0; i < nc; i++) {
        cell_depth[i] = cs.v[i].depth;
        cell_body_off[i] = cs.v[i].body_off;
        cell_body_num[i] = cs.v[i].body_num;
        cell_center[3 * i] = cs.v[i].c[0];
        cell_center[3 * i + 1] = cs.v[i].c[1];
        cell_center[3 * i + 2] = cs.v[i].c[2];
    }
    free(cs.v);
    return nc;
}

/* Interaction lists of the reference traversal, grouped by ascending target.
 * Two-call protocol: call with NULL outputs to get the counts. */
static zlist g_last_p2p, g_last_m2l;

int z64_lists(int max_depth, int images, double cycle, double theta, long* n_p2p, long* n_m2l)
{
    double center[3] = {cycle / 2, cycle / 2, cycle / 2};
    zcells cs = {0, 0, NULL};
    int dummy = 0;
    build_tree(0, NULL, cycle / 2, center, max_depth, &cs, &dummy);
    ztrav t;
    int nimg;
    traverse(&cs, theta, images, cycle, &t, &nimg);
    free(g_last_p2p.tgt); free(g_last_p2p.src); free(g_last_p2p.off);
    free(g_last_m2l.tgt); free(g_last_m2l.src); free(g_last_m2l.off);
    g_last_p2p = t.p2p;
    g_last_m2l = t.m2l;
    *n_p2p = t.p2p.n;
    *n_m2l = t.m2l.n;
    free(cs.v);
    return nimg;
}

void z64_lists_fetch(int which, int* tgt, int* src, double* off)
{
    zlist* l = which == 0 ? &g_last_p2p : &g_last_m2l;
    memcpy(tgt, l->tgt, sizeof(int) * l->n);
    memcpy(src, l->src, sizeof(int) * l->n);
    memcpy(off, l->off, sizeof(double) * 3 * l->n);
}

/* Full FMM as GPUSolver::solve + dipole_correction + get_result(sort) would compute it.
 * xyz: 3n doubles (converted from float by the caller, as zeta_fmm_solver.cpp:26-35 does),
 * q: n doubles.  Outputs in input order: pot[n] (kJ/mol/e), force[3n] (kJ/mol/nm), energy.
 * stage_mask bit0: far field (P2M..L2P), bit1: near field (P2P), bit2: dipole correction. */
int z64_solve(int n, const double* xyz, const double* q, double cycle, int P, int max_depth, int images,
              double theta, int stage_mask, double* pot, double* force, double* energy)
{
    if (P < 0 || P > 40 || max_depth < 0 || max_depth > 9 || images < 0 || n < 0) return -1;
    set_omp();
    double box_r = cycle / 2;
    double center[3] = {cycle / 2, cycle / 2, cycle / 2};
    int* order = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    zcells cs = {0, 0, NULL};
    build_tree(n, xyz, box_r, center, max_depth, &cs, order);
    ztrav tr;
    int nimg;
    traverse(&cs, theta, images, cycle, &tr, &nimg);
    int ncell = cs.ncell;
    int np = npack(P);
    int ny = (P + 1) * (P + 1);
    zc* Ms = (zc*)calloc((size_t)ncell * np, sizeof(zc));
    zc* Ls = (zc*)calloc((size_t)ncell * np, sizeof(zc));
    /* sorted bodies */
    double* bx = (double*)malloc(sizeof(double) * 3 * (n > 0 ? n : 1));
    double* bq = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    double* bp = (double*)calloc(n > 0 ? n : 1, sizeof(double));
    double* bf = (double*)calloc(3 * (n > 0 ? n : 1), sizeof(double));
    for (int i = 0; i < n; i++) {
        int s = order[i];
        bx[3 * i] = xyz[3 * s]; bx[3 * i + 1] = xyz[3 * s + 1]; bx[3 * i + 2] = xyz[3 * s + 2];
        bq[i] = q[s];
    }
    int ntree = ncell - nimg;
    int real_max_depth = 0;
    for (int i = 0; i < ntree; i++) if (cs.v[i].depth > real_max_depth) real_max_depth = cs.v[i].depth;

    if (stage_mask & 1) {
        /* P2M over leaves */
#pragma omp parallel
        {
            zc* Y = (zc*)malloc(sizeof(zc) * ny);
#pragma omp for schedule(dynamic, 16)
            for (int c = 0; c < ntree; c++) {
                zcell* C = &cs.v[c];
                if (C->depth != real_max_depth) continue;
                for (int i = 0; i < C->body_num; i++) {
                    int b = C->body_off + i;
                    double d[3] = {bx[3 * b] - C->c[0], bx[3 * b + 1] - C->c[1], bx[3 * b + 2] - C->c[2]};
                    op_p2m(P, Y, d, bq[b], Ms + (size_t)c * np);
                }
            }
            free(Y);
        }
        /* M2M from max-depth-1 up to 0 (kernel.cu:857-861) */
        for (int lev = real_max_depth - 1; lev >= 0; lev--) {
#pragma omp parallel
            {
                zc* Y = (zc*)malloc(sizeof(zc) * ny);
#pragma omp for schedule(dynamic, 4)
                for (int c = 0; c < ntree; c++) {
                    zcell* C = &cs.v[c];
                    if (C->depth != lev) continue;
                    for (int i = 0; i < C->child_num; i++) {
                        int ch = C->child_off + i;
                        zcell* H = &cs.v[ch];
                        double d[3] = {C->c[0] - H->c[0], C->c[1] - H->c[1], C->c[2] - H->c[2]};
                        op_m2m(P, Y, d, Ms + (size_t)ch * np, Ms + (size_t)c * np);
                    }
                }
                free(Y);
            }
        }
        /* image M2M (kernel.cu:864-869): image cell i from its child, 27 shifts of cycle*3^i */
        {
            zc* Y = (zc*)malloc(sizeof(zc) * ny);
            double cyc = cycle;
            for (int i = 0; i < nimg - 1; i++) {
                int c = ntree + i;
                zcell* C = &cs.v[c];
                zcell* H = &cs.v[C->child_off];
                for (int pz = -1; pz <= 1; pz++)
                    for (int py = -1; py <= 1; py++)
                        for (int px = -1; px <= 1; px++) {
                            double d[3] = {C->c[0] - H->c[0] - px * cyc, C->c[1] - H->c[1] - py * cyc,
                                           C->c[2] - H->c[2] - pz * cyc};
                            op_m2m(P, Y, d, Ms + (size_t)C->child_off * np, Ms + (size_t)c * np);
                        }
                cyc *= 3;
            }
            free(Y);
        }
        /* M2L, grouped by target (kernel.cu:872) */
        {
            long ne = tr.m2l.n;
            /* target row starts */
            long* row = (long*)malloc(sizeof(long) * (ne + 1));
            long nrow = 0;
            for (long e = 0; e < ne; e++)
                if (e == 0 || tr.m2l.tgt[e] != tr.m2l.tgt[e - 1]) row[nrow++] = e;
            row[nrow] = ne;
#pragma omp parallel
            {
                zc* Y = (zc*)malloc(sizeof(zc) * ny);
#pragma omp for schedule(dynamic, 4)
                for (long r = 0; r < nrow; r++) {
                    for (long e = row[r]; e < row[r + 1]; e++) {
                        int tc = tr.m2l.tgt[e], sc = tr.m2l.src[e];
                        const double* o = &tr.m2l.off[3 * e];
                        double d[3] = {cs.v[tc].c[0] - (cs.v[sc].c[0] + o[0]), cs.v[tc].c[1] - (cs.v[sc].c[1] + o[1]),
                                       cs.v[tc].c[2] - (cs.v[sc].c[2] + o[2])};
                        op_m2l(P, Y, d, Ms + (size_t)sc * np, Ls + (size_t)tc * np);
                    }
                }
                free(Y);
            }
            free(row);
        }
        /* L2L from depth 0 down (kernel.cu:885-889) */
        for (int lev = 0; lev < real_max_depth; lev++) {
#pragma omp parallel
            {
                zc* Y = (zc*)malloc(sizeof(zc) * ny);
#pragma omp for schedule(dynamic, 4)
                for (int c = 0; c < ntree; c++) {
                    zcell* C = &cs.v[c];
                    if (C->depth != lev) continue;
                    for (int i = 0; i < C->child_num; i++) {
                        int ch = C->child_off + i;
                        zcell* H = &cs.v[ch];
                        double d[3] = {H->c[0] - C->c[0], H->c[1] - C->c[1], H->c[2] - C->c[2]};
                        op_l2l(P, Y, d, Ls + (size_t)c * np, Ls + (size_t)ch * np);
                    }
                }
                free(Y);
            }
        }
        /* L2P */
#pragma omp parallel
        {
            zc* Y = (zc*)malloc(sizeof(zc) * ny);
            zc* YD = (zc*)malloc(sizeof(zc) * ny);
#pragma omp for schedule(dynamic, 16)
            for (int c = 0; c < ntree; c++) {
                zcell* C = &cs.v[c];
                if (C->depth != real_max_depth) continue;
                for (int i = 0; i < C->body_num; i++) {
                    int b = C->body_off + i;
                    double d[3] = {bx[3 * b] - C->c[0], bx[3 * b + 1] - C->c[1], bx[3 * b + 2] - C->c[2]};
                    op_l2p(P, Y, YD, d, Ls + (size_t)c * np, &bp[b], &bf[3 * b]);
                }
            }
            free(Y);
            free(YD);
        }
    }
    if (stage_mask & 2) {
        /* P2P (kernel.cu:456-496), rows grouped by target */
        long ne = tr.p2p.n;
        long* row = (long*)malloc(sizeof(long) * (ne + 1));
        long nrow = 0;
        for (long e = 0; e < ne; e++)
            if (e == 0 || tr.p2p.tgt[e] != tr.p2p.tgt[e - 1]) row[nrow++] = e;
        row[nrow] = ne;
#pragma omp parallel for schedule(dynamic, 4)
        for (long r = 0; r < nrow; r++) {
            for (long e = row[r]; e < row[r + 1]; e++) {
                zcell* T = &cs.v[tr.p2p.tgt[e]];
                zcell* S = &cs.v[tr.p2p.src[e]];
                const double* o = &tr.p2p.off[3 * e];
                for (int i = T->body_off; i < T->body_off + T->body_num; i++) {
                    double p = 0, f0 = 0, f1 = 0, f2 = 0;
                    for (int j = S->body_off; j < S->body_off + S->body_num; j++) {
                        double d0 = bx[3 * i] - (bx[3 * j] + o[0]);
                        double d1 = bx[3 * i + 1] - (bx[3 * j + 1] + o[1]);
                        double d2 = bx[3 * i + 2] - (bx[3 * j + 2] + o[2]);
                        double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                        if (r > 0) {
                            p += bq[j] / r;
                            double s = bq[j] / r / r / r;
                            f0 += s * -d0; f1 += s * -d1; f2 += s * -d2;
                        }
                    }
                    bp[i] += p;
                    bf[3 * i] += f0; bf[3 * i + 1] += f1; bf[3 * i + 2] += f2;
                }
            }
        }
        free(row);
    }
    /* -E -> F and unit conversion (gpu_solver.cu:250-256) */
    for (int i = 0; i < n; i++) {
        bp[i] *= KE_GMX;
        bf[3 * i] *= -bq[i] * KE_GMX;
        bf[3 * i + 1] *= -bq[i] * KE_GMX;
        bf[3 * i + 2] *= -bq[i] * KE_GMX;
    }
    /* dipole correction (solver.cpp:30-49), over the sorted bodies */
    if (stage_mask & 4) {
        double coef = 4 * M_PI / (3 * cycle * cycle * cycle);
        double dip[3] = {0, 0, 0};
        for (int i = 0; i < n; i++) {
            dip[0] += bx[3 * i] * bq[i];
            dip[1] += bx[3 * i + 1] * bq[i];
            dip[2] += bx[3 * i + 2] * bq[i];
        }
        double dn = dip[0] * dip[0] + dip[1] * dip[1] + dip[2] * dip[2];
        for (int i = 0; i < n; i++) {
            bp[i] -= coef * dn / n / bq[i] * KE_GMX;
            bf[3 * i] += coef * dip[0] * bq[i] * KE_GMX;
            bf[3 * i + 1] += coef * dip[1] * bq[i] * KE_GMX;
            bf[3 * i + 2] += coef * dip[2] * bq[i] * KE_GMX;
        }
    }
    /* back to input order (solver.cpp:58-67), energy 0.5*sum(q*phi) (fmm.cpp:89-98) */
    double e = 0;
    for (int i = 0; i < n; i++) {
        int s = order[i];
        pot[s] = bp[i];
        force[3 * s] = bf[3 * i];
        force[3 * s + 1] = bf[3 * i + 1];
        force[3 * s + 2] = bf[3 * i + 2];
        e += bp[i] * bq[i];
    }
    *energy = e / 2;
    free(order); free(cs.v); free(Ms); free(Ls); free(bx); free(bq); free(bp); free(bf);
    free(tr.p2p.tgt); free(tr.p2p.src); free(tr.p2p.off);
    free(tr.m2l.tgt); free(tr.m2l.src); free(tr.m2l.off);
    return 0;
}

/* ---------------------------------------------------------------- harmonics probes */

/* Exposes the three harmonic recurrences for unit tests of the library's own
 * (Cartesian) harmonics and operator matrices. out: 2*(P+1)^2 doubles. */
void z64_harmonics(int kind, int P, const double d[3], double* out)
{
    double rho, th, ph;
    to_sph(d, &rho, &th, &ph);
    int ny = (P + 1) * (P + 1);
    zc* Y = (zc*)calloc(ny, sizeof(zc));
    if (kind == 0) harm_regular(Y, P, rho, th, ph);
    else if (kind == 1) harm_regular_dtheta(Y, P, rho, th, ph);
    else harm_singular(Y, P, rho, th, ph);
    for (int i = 0; i < ny; i++) { out[2 * i] = Y[i].re; out[2 * i + 1] = Y[i].im; }
    free(Y);
}

/* Single operator applications on packed complex expansions (2*npack doubles). */
void z64_apply(int kind, int P, const double d[3], const double* in, double* out)
{
    int ny = (P + 1) * (P + 1);
    zc* Y = (zc*)calloc(ny, sizeof(zc));
    const zc* a = (const zc*)in;
    zc* b = (zc*)out;
    if (kind == 0) op_m2m(P, Y, d, a, b);
    else if (kind == 1) op_l2l(P, Y, d, a, b);
    else op_m2l(P, Y, d, a, b);
    free(Y);
}
