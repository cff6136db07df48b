// Host FP64 construction of translation operators, stencils and reference lists.
//
// The operators restate the exafmm-style solid-harmonic translations of the
// reference GPU solver (src/gromacs/zeta_fmm/kernel.cu) as real matrices acting
// on the (P+1)^2 real representation of an expansion:
//   M2M  kernel.cu:325-351   L2L  kernel.cu:422-451   M2L  kernel.cu:572-603
// including the reference's j+n<=P truncation of M2L (kernel.cu:585).  Every
// complex term "out(j,k) += c * [conj] in(n,m) * Y(a,b)" of those loops becomes
// four real matrix entries, so the matrices are the exact linear maps of the
// reference loops.  The harmonics are evaluated with Cartesian recurrences of the
// same normalisation (Y_n^m = (-1)^n r^n P_n^m e^{im phi}/(n+m)!, singular
// S_n^m = (-1)^n (n-m)! P_n^m e^{im phi}/r^(n+1)) instead of the reference's
// spherical-angle recurrences.
#include "operators.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

#include "common.cuh"

namespace gbfmm {

static inline int pk(int n, int m) { return n * (n + 1) / 2 + m; }
static inline int sgn(int n) { return (n & 1) ? -1 : 1; }

void harm_regular(int P, const double d[3], double* re, double* im)
{
    const double x = d[0], y = d[1], z = d[2], r2 = x * x + y * y + z * z;
    double sr = 1, si = 0;
    for (int m = 0; m <= P; m++) {
        if (m > 0) {
            double tr = (sr * x - si * y) / (2 * m), ti = (sr * y + si * x) / (2 * m);
            sr = tr;
            si = ti;
        }
        re[pk(m, m)] = sr;
        im[pk(m, m)] = si;
        if (m + 1 <= P) {
            re[pk(m + 1, m)] = -z * sr;
            im[pk(m + 1, m)] = -z * si;
        }
        for (int n = m + 1; n < P; n++) {
            double c = 1.0 / ((n + m + 1.0) * (n - m + 1.0));
            re[pk(n + 1, m)] = -((2 * n + 1) * z * re[pk(n, m)] + r2 * re[pk(n - 1, m)]) * c;
            im[pk(n + 1, m)] = -((2 * n + 1) * z * im[pk(n, m)] + r2 * im[pk(n - 1, m)]) * c;
        }
    }
}

void harm_singular(int P, const double d[3], double* re, double* im)
{
    const double x = d[0], y = d[1], z = d[2], r2 = x * x + y * y + z * z;
    const double ir2 = 1.0 / r2;
    double sr = 1.0 / std::sqrt(r2), si = 0;
    for (int m = 0; m <= P; m++) {
        if (m > 0) {
            double f = (2 * m - 1) * ir2;
            double tr = (sr * x - si * y) * f, ti = (sr * y + si * x) * f;
            sr = tr;
            si = ti;
        }
        re[pk(m, m)] = sr;
        im[pk(m, m)] = si;
        if (m + 1 <= P) {
            re[pk(m + 1, m)] = -(2 * m + 1) * z * sr * ir2;
            im[pk(m + 1, m)] = -(2 * m + 1) * z * si * ir2;
        }
        for (int n = m + 1; n < P; n++) {
            double a = (2 * n + 1) * z, b = (double)(n * n - m * m);
            re[pk(n + 1, m)] = -(a * re[pk(n, m)] + b * re[pk(n - 1, m)]) * ir2;
            im[pk(n + 1, m)] = -(a * im[pk(n, m)] + b * im[pk(n - 1, m)]) * ir2;
        }
    }
}

namespace {

// Harmonic table with access to negative m through conjugate symmetry.
struct Harm {
    int P;
    std::vector<double> re, im;
    Harm(int P_, const double d[3], bool singular) : P(P_), re((P_ + 1) * (P_ + 2) / 2), im((P_ + 1) * (P_ + 2) / 2)
    {
        if (singular) harm_singular(P, d, re.data(), im.data());
        else harm_regular(P, d, re.data(), im.data());
    }
    void get(int n, int m, double& yr, double& yi) const
    {
        if (m >= 0) {
            yr = re[pk(n, m)];
            yi = im[pk(n, m)];
        } else {
            yr = re[pk(n, -m)];
            yi = -im[pk(n, -m)];
        }
    }
};

// out(j,k) += c * [conj](in(n,m)) * (yr + i yi), as real matrix entries.
struct RMat {
    int R;
    double* a;
    void add(int r, int c, double v) { a[(size_t)r * R + c] += v; }
    void term(int j, int k, int n, int m, bool conj_in, double c, double yr, double yi)
    {
        int rr = ridx_re(j, k), ri = k > 0 ? ridx_im(j, k) : -1;
        int cr = ridx_re(n, m), ci = m > 0 ? ridx_im(n, m) : -1;
        if (!conj_in) {
            add(rr, cr, c * yr);
            if (ci >= 0) add(rr, ci, -c * yi);
            if (ri >= 0) {
                add(ri, cr, c * yi);
                if (ci >= 0) add(ri, ci, c * yr);
            }
        } else {
            add(rr, cr, c * yr);
            if (ci >= 0) add(rr, ci, c * yi);
            if (ri >= 0) {
                add(ri, cr, c * yi);
                if (ci >= 0) add(ri, ci, -c * yr);
            }
        }
    }
};

}  // namespace

void m2m_matrix(int P, const double dx[3], double* A)
{
    const int R = nreal(P);
    std::memset(A, 0, sizeof(double) * R * R);
    Harm Y(P, dx, false);
    RMat M{R, A};
    double yr, yi;
    for (int j = 0; j <= P; j++)
        for (int k = 0; k <= j; k++)
            for (int n = 0; n <= j; n++) {
                int lo = std::max(-n, -j + k + n), hi = std::min(k - 1, n);
                for (int m = lo; m <= hi; m++) {
                    Y.get(n, -m, yr, yi);
                    int c = (m >= 0 ? 1 : sgn(m)) * sgn(n);
                    M.term(j, k, j - n, k - m, false, c, yr, yi);
                }
                int hi2 = std::min(n, j + k - n);
                for (int m = k; m <= hi2; m++) {
                    Y.get(n, -m, yr, yi);
                    M.term(j, k, j - n, m - k, true, sgn(k + n + m), yr, yi);
                }
            }
}

void l2l_matrix(int P, const double dX[3], double* A)
{
    const int R = nreal(P);
    std::memset(A, 0, sizeof(double) * R * R);
    Harm Y(P, dX, false);
    RMat M{R, A};
    double yr, yi;
    for (int j = 0; j <= P; j++)
        for (int k = 0; k <= j; k++)
            for (int n = j; n <= P; n++) {
                for (int m = j + k - n; m < 0; m++) {
                    Y.get(n - j, m - k, yr, yi);
                    M.term(j, k, n, -m, true, sgn(k), yr, yi);
                }
                for (int m = 0; m <= n; m++) {
                    if (n - j >= std::abs(m - k)) {
                        Y.get(n - j, m - k, yr, yi);
                        M.term(j, k, n, m, false, sgn((m - k) * (m < k)), yr, yi);
                    }
                }
            }
}

void m2l_matrix(int P, const double dX[3], double* A)
{
    const int R = nreal(P);
    std::memset(A, 0, sizeof(double) * R * R);
    Harm S(P, dX, true);
    RMat M{R, A};
    double yr, yi;
    for (int j = 0; j <= P; j++) {
        int cnm = sgn(j);
        for (int k = 0; k <= j; k++)
            for (int n = 0; n + j <= P; n++) {
                for (int m = -n; m < 0; m++) {
                    S.get(j + n, m - k, yr, yi);
                    M.term(j, k, n, -m, true, cnm, yr, yi);
                }
                for (int m = 0; m <= n; m++) {
                    S.get(j + n, m - k, yr, yi);
                    M.term(j, k, n, m, false, cnm * sgn((k - m) * (k < m) + m), yr, yi);
                }
            }
    }
}

// ------------------------------------------------------------------ scaled operators

void scaled_m2m(int P, int o, double* A)
{
    const int R = nreal(P);
    double dx[3] = {-(((o >> 2) & 1) ? 0.5 : -0.5), -(((o >> 1) & 1) ? 0.5 : -0.5), -((o & 1) ? 0.5 : -0.5)};
    m2m_matrix(P, dx, A);
    for (int r = 0; r < R; r++) {
        double s = std::ldexp(1.0, -rdeg(r));
        for (int c = 0; c < R; c++) A[(size_t)r * R + c] *= s;
    }
}

void scaled_l2l(int P, int o, double* A)
{
    const int R = nreal(P);
    double dX[3] = {((o >> 2) & 1) ? 0.5 : -0.5, ((o >> 1) & 1) ? 0.5 : -0.5, (o & 1) ? 0.5 : -0.5};
    l2l_matrix(P, dX, A);
    for (int c = 0; c < R; c++) {
        double s = std::ldexp(1.0, -(rdeg(c) + 1));
        for (int r = 0; r < R; r++) A[(size_t)r * R + c] *= s;
    }
}

void scaled_m2l(int P, const M2LClass& cl, double* A)
{
    const int R = nreal(P);
    double d[3];
    for (int i = 0; i < 3; i++) d[i] = cl.kind == 0 ? (double)cl.v[i] : 0.5 * cl.v[i];
    m2l_matrix(P, d, A);
    if (cl.kind == 1) {
        for (int c = 0; c < R; c++) {
            double s = std::ldexp(1.0, rdeg(c));
            for (int r = 0; r < R; r++) A[(size_t)r * R + c] *= s;
        }
    }
}

static void matmul(int R, const double* A, const double* B, double* C)
{
    std::vector<double> t((size_t)R * R, 0.0);
    for (int i = 0; i < R; i++)
        for (int k = 0; k < R; k++) {
            double a = A[(size_t)i * R + k];
            if (a == 0) continue;
            for (int j = 0; j < R; j++) t[(size_t)i * R + j] += a * B[(size_t)k * R + j];
        }
    std::memcpy(C, t.data(), sizeof(double) * R * R);
}

// Image levels of the reference: M2M of the image cells (kernel.cu:356-406,
// launched at :864-869) and the 26x27 M2L entries per level into the root
// (traverser.cpp:162-214), composed into one linear map of the root multipole.
void lattice_operator(int P, int images, double* A)
{
    const int R = nreal(P);
    std::memset(A, 0, sizeof(double) * R * R);
    if (images < 2) return;
    std::vector<double> C((size_t)R * R, 0.0), S((size_t)R * R), T((size_t)R * R), B((size_t)R * R), tmp((size_t)R * R);
    for (int i = 0; i < R; i++) C[(size_t)i * R + i] = 1.0;
    double c3 = 1.0;
    for (int m = 0; m < images - 1; m++) {
        std::fill(S.begin(), S.end(), 0.0);
        for (int pz = -1; pz <= 1; pz++)
            for (int py = -1; py <= 1; py++)
                for (int px = -1; px <= 1; px++) {
                    if (px == 0 && py == 0 && pz == 0) continue;
                    for (int cz = -1; cz <= 1; cz++)
                        for (int cy = -1; cy <= 1; cy++)
                            for (int cx = -1; cx <= 1; cx++) {
                                double d[3] = {-(px * 3 + cx) * c3, -(py * 3 + cy) * c3, -(pz * 3 + cz) * c3};
                                m2l_matrix(P, d, T.data());
                                for (size_t i = 0; i < S.size(); i++) S[i] += T[i];
                            }
                }
        matmul(R, S.data(), C.data(), tmp.data());
        for (size_t i = 0; i < (size_t)R * R; i++) A[i] += tmp[i];
        if (m < images - 2) {
            std::fill(B.begin(), B.end(), 0.0);
            for (int pz = -1; pz <= 1; pz++)
                for (int py = -1; py <= 1; py++)
                    for (int px = -1; px <= 1; px++) {
                        double d[3] = {-px * c3, -py * c3, -pz * c3};
                        m2m_matrix(P, d, T.data());
                        for (size_t i = 0; i < B.size(); i++) B[i] += T[i];
                    }
            matmul(R, B.data(), C.data(), C.data());
        }
        c3 *= 3.0;
    }
}

// The lattice operator weighted by the image index of each source box: three
// R x R FP64 matrices A_a (a = x, y, z) with L~_a = A_a M~_root the local
// expansion, at the root, of the field of every far image box n weighted by
// n_a (in periods).  Same hierarchy as lattice_operator: a level-m supercell
// holds 3^m boxes per axis; with C_m its multipole operator, its first moment
// C^a_m = sum over its boxes of (box offset from the supercell centre)_a x the
// box's M2M satisfies C^a_{m+1} = sum_p M2M(p 3^m) (C^a_m + p_a 3^m C_m); a
// source supercell centred at offset o contributes M2L (C^a_m + o_a C_m).  Used
// by the virial's image-shift term.
void lattice_shift_operators(int P, int images, double* A3)
{
    const int R = nreal(P);
    const size_t RR = (size_t)R * R;
    std::memset(A3, 0, sizeof(double) * 3 * RR);
    if (images < 2) return;
    // per level: S = sum of the source M2L operators and Sa = sum of o_a times
    // them, so that sum T (C^a + o_a C) = S C^a + Sa C; likewise for the M2M step
    std::vector<double> C(RR, 0.0), Ca[3], T(RR), S(RR), Sa[3], tmp(RR), B(RR), Ba[3], Cn(RR), Can[3];
    for (int a = 0; a < 3; a++) {
        Ca[a].assign(RR, 0.0);
        Sa[a].assign(RR, 0.0);
        Ba[a].assign(RR, 0.0);
        Can[a].assign(RR, 0.0);
    }
    for (int i = 0; i < R; i++) C[(size_t)i * R + i] = 1.0;
    double c3 = 1.0;
    for (int m = 0; m < images - 1; m++) {
        std::fill(S.begin(), S.end(), 0.0);
        for (int a = 0; a < 3; a++) std::fill(Sa[a].begin(), Sa[a].end(), 0.0);
        for (int pz = -1; pz <= 1; pz++)
            for (int py = -1; py <= 1; py++)
                for (int px = -1; px <= 1; px++) {
                    if (px == 0 && py == 0 && pz == 0) continue;
                    for (int cz = -1; cz <= 1; cz++)
                        for (int cy = -1; cy <= 1; cy++)
                            for (int cx = -1; cx <= 1; cx++) {
                                const double o[3] = {(px * 3 + cx) * c3, (py * 3 + cy) * c3, (pz * 3 + cz) * c3};
                                const double d[3] = {-o[0], -o[1], -o[2]};
                                m2l_matrix(P, d, T.data());
                                for (size_t i = 0; i < RR; i++) {
                                    S[i] += T[i];
                                    for (int a = 0; a < 3; a++) Sa[a][i] += o[a] * T[i];
                                }
                            }
                }
        for (int a = 0; a < 3; a++) {
            matmul(R, S.data(), Ca[a].data(), tmp.data());
            for (size_t i = 0; i < RR; i++) A3[a * RR + i] += tmp[i];
            matmul(R, Sa[a].data(), C.data(), tmp.data());
            for (size_t i = 0; i < RR; i++) A3[a * RR + i] += tmp[i];
        }
        if (m < images - 2) {
            std::fill(B.begin(), B.end(), 0.0);
            for (int a = 0; a < 3; a++) std::fill(Ba[a].begin(), Ba[a].end(), 0.0);
            for (int pz = -1; pz <= 1; pz++)
                for (int py = -1; py <= 1; py++)
                    for (int px = -1; px <= 1; px++) {
                        const double p[3] = {px * c3, py * c3, pz * c3};
                        const double d[3] = {-p[0], -p[1], -p[2]};
                        m2m_matrix(P, d, T.data());
                        for (size_t i = 0; i < RR; i++) {
                            B[i] += T[i];
                            for (int a = 0; a < 3; a++) Ba[a][i] += p[a] * T[i];
                        }
                    }
            for (int a = 0; a < 3; a++) {
                matmul(R, B.data(), Ca[a].data(), Can[a].data());
                matmul(R, Ba[a].data(), C.data(), tmp.data());
                for (size_t i = 0; i < RR; i++) Can[a][i] += tmp[i];
            }
            matmul(R, B.data(), C.data(), Cn.data());
            C = Cn;
            for (int a = 0; a < 3; a++) Ca[a] = Can[a];
        }
        c3 *= 3.0;
    }
}

// ------------------------------------------------------------------ stencils

Stencils build_stencils(double theta)
{
    Stencils st;
    std::map<std::tuple<int, int, int, int>, int> cls_id;
    auto class_of = [&](int kind, int a, int b, int c) {
        auto key = std::make_tuple(kind, a, b, c);
        auto it = cls_id.find(key);
        if (it != cls_id.end()) return it->second;
        int id = (int)st.classes.size();
        st.classes.push_back(M2LClass{kind, {a, b, c}});
        cls_id[key] = id;
        return id;
    };
    // near test exactly as NearFieldSelector::is_near (traverser.cpp:14-21) on unit geometry
    auto near_same = [&](int a, int b, int c) {
        double r = std::sqrt((double)(a * a + b * b + c * c)) * theta;
        return !(r > 1.0);  // r_a + r_b = 0.5 + 0.5
    };
    auto near_mixed = [&](int a, int b, int c) {  // Delta = w/2, radii 0.5 + 1
        double r = std::sqrt(0.25 * (a * a + b * b + c * c)) * theta;
        return !(r > 1.5);
    };
    for (int lt = 0; lt < 2; lt++) {
        // near set of the parent: root shifts (level 1) or the same-level near set
        std::vector<std::array<int, 3>> nset;
        for (int z = -3; z <= 3; z++)
            for (int y = -3; y <= 3; y++)
                for (int x = -3; x <= 3; x++) {
                    if (lt == 0) {
                        if (std::abs(x) <= 1 && std::abs(y) <= 1 && std::abs(z) <= 1) nset.push_back({x, y, z});
                    } else if (near_same(x, y, z)) {
                        nset.push_back({x, y, z});
                    }
                }
        for (int s = 0; s < 8; s++) {
            int o[3] = {(s >> 2) & 1, (s >> 1) & 1, s & 1};
            for (auto& m : nset) {
                int w[3];
                for (int i = 0; i < 3; i++) w[i] = 2 * o[i] - 4 * m[i] - 1;
                if (!near_mixed(w[0], w[1], w[2])) {
                    StencilEntry e;
                    e.mode = 1;
                    e.d[0] = m[0]; e.d[1] = m[1]; e.d[2] = m[2];
                    e.cls = class_of(1, w[0], w[1], w[2]);
                    st.m2l[lt][s].push_back(e);
                } else {
                    for (int ob = 0; ob < 8; ob++) {
                        int b[3] = {(ob >> 2) & 1, (ob >> 1) & 1, ob & 1};
                        int n[3];
                        for (int i = 0; i < 3; i++) n[i] = o[i] - b[i] - 2 * m[i];
                        if (!near_same(n[0], n[1], n[2])) {
                            StencilEntry e;
                            e.mode = 0;
                            e.d[0] = -n[0]; e.d[1] = -n[1]; e.d[2] = -n[2];
                            e.cls = class_of(0, n[0], n[1], n[2]);
                            st.m2l[lt][s].push_back(e);
                        }
                    }
                }
            }
        }
    }
    for (int z = -3; z <= 3; z++)
        for (int y = -3; y <= 3; y++)
            for (int x = -3; x <= 3; x++)
                if (near_same(x, y, z)) {
                    st.p2p.push_back(x);
                    st.p2p.push_back(y);
                    st.p2p.push_back(z);
                }
    return st;
}

// ------------------------------------------------------------------ packing

PackPlan make_pack_plan(int P, OpType t)
{
    PackPlan pl;
    pl.P = P;
    pl.R = nreal(P);
    pl.nblk = (pl.R + 7) / 8;
    pl.c0.resize(pl.nblk);
    pl.c1.resize(pl.nblk);
    pl.off.resize(pl.nblk);
    int off = 0;
    for (int b = 0; b < pl.nblk; b++) {
        int lo = pl.R, hi = 0;
        for (int r = 8 * b; r < std::min(pl.R, 8 * b + 8); r++) {
            int j = rdeg(r), a, z;
            if (t == OP_M2L) { a = 0; z = (P - j + 1) * (P - j + 1); }
            else if (t == OP_M2M) { a = 0; z = (j + 1) * (j + 1); }
            else { a = j * j; z = pl.R; }
            lo = std::min(lo, a);
            hi = std::max(hi, z);
        }
        pl.c0[b] = lo;
        pl.c1[b] = hi;
        pl.off[b] = off;
        off += 8 * (hi - lo);
    }
    pl.packed = off;
    return pl;
}

void pack_operator(const PackPlan& pl, const double* A, float* out)
{
    for (int b = 0; b < pl.nblk; b++)
        for (int c = pl.c0[b]; c < pl.c1[b]; c++)
            for (int i = 0; i < 8; i++) {
                int r = 8 * b + i;
                out[pl.off[b] + (c - pl.c0[b]) * 8 + i] = r < pl.R ? (float)A[(size_t)r * pl.R + c] : 0.0f;
            }
}

// Splits the row blocks into 'groups' contiguous row ranges of about equal work
// (one CTA per group and target tile), then, inside each group, cuts blocks into
// column pieces no larger than the per-warp share and assigns the pieces to warps
// longest-first, at most max_items per warp.  Returns false if that cap cannot
// be met.
bool make_work_items(const PackPlan& pl, int n_warps, int groups, int max_items, WorkPartition& out)
{
    out = WorkPartition();
    out.groups = groups;
    long total = 0;
    for (int b = 0; b < pl.nblk; b++) total += pl.c1[b] - pl.c0[b];
    // contiguous block ranges per group
    std::vector<int> gb(groups + 1, pl.nblk);
    gb[0] = 0;
    {
        long acc = 0;
        int g = 1;
        for (int b = 0; b < pl.nblk && g < groups; b++) {
            acc += pl.c1[b] - pl.c0[b];
            if (acc * groups >= total * g) gb[g++] = b + 1;
        }
        for (; g < groups; g++) gb[g] = pl.nblk;
    }
    for (int g = 0; g < groups; g++) {
        out.row0.push_back(8 * gb[g]);
        out.row1.push_back(std::min(pl.R, 8 * gb[g + 1]));
        long gw = 0;
        for (int b = gb[g]; b < gb[g + 1]; b++) gw += pl.c1[b] - pl.c0[b];
        long share = std::max<long>(1, (gw + n_warps - 1) / n_warps);
        std::vector<WorkItem> pieces;
        for (int b = gb[g]; b < gb[g + 1]; b++)
            for (int c = pl.c0[b]; c < pl.c1[b]; c += (int)share) {
                WorkItem it;
                it.blk = (int16_t)b;
                it.ca = (int16_t)c;
                it.cb = (int16_t)std::min<long>(pl.c1[b], c + share);
                it.pad = 0;
                pieces.push_back(it);
            }
        std::stable_sort(pieces.begin(), pieces.end(),
                         [](const WorkItem& x, const WorkItem& y) { return (x.cb - x.ca) > (y.cb - y.ca); });
        std::vector<std::vector<WorkItem>> per(n_warps);
        std::vector<long> load(n_warps, 0);
        for (const WorkItem& it : pieces) {
            int best = -1;
            for (int w = 0; w < n_warps; w++)
                if ((int)per[w].size() < max_items && (best < 0 || load[w] < load[best])) best = w;
            if (best < 0) return false;
            per[best].push_back(it);
            load[best] += it.cb - it.ca;
        }
        for (int w = 0; w < n_warps; w++) {
            out.warp_begin.push_back((int)out.items.size());
            for (const WorkItem& it : per[w]) out.items.push_back(it);
        }
        out.warp_begin.push_back((int)out.items.size());
    }
    return true;
}

// ------------------------------------------------------------------ reference lists

void emit_lists(const Stencils& st, int D, int images, RefLists& p2p, RefLists& m2l)
{
    p2p = RefLists();
    m2l = RefLists();
    const bool periodic = images > 0;
    const long ntree = level_base(D + 1);
    struct E { long key; int src, ox, oy, oz; };
    std::vector<E> buf;
    auto pidx = [](int px, int py, int pz) { return (pz + 1) * 9 + (py + 1) * 3 + (px + 1); };
    auto floordiv = [](int a, int n) { return a >= 0 ? a / n : -((-a + n - 1) / n); };

    // root row: far lattice entries (traverser.cpp:174-211)
    if (images >= 2) {
        long pw = 1;
        for (int m = 0; m < images - 1; m++) {
            int src = m == 0 ? 0 : (int)(ntree + m - 1);
            for (int pz = -1; pz <= 1; pz++)
                for (int py = -1; py <= 1; py++)
                    for (int px = -1; px <= 1; px++) {
                        if (!px && !py && !pz) continue;
                        for (int cz = -1; cz <= 1; cz++)
                            for (int cy = -1; cy <= 1; cy++)
                                for (int cx = -1; cx <= 1; cx++) {
                                    m2l.tgt.push_back(0);
                                    m2l.src.push_back(src);
                                    m2l.off.push_back((int)((px * 3 + cx) * pw));
                                    m2l.off.push_back((int)((py * 3 + cy) * pw));
                                    m2l.off.push_back((int)((pz * 3 + cz) * pw));
                                }
                    }
            pw *= 3;
        }
    }
    for (int k = 1; k <= D; k++) {
        const int nk = 1 << k, nk1 = 1 << (k - 1);
        const int lt = k == 1 ? 0 : 1;
        const long ncell = 1L << (3 * k);
        for (long code = 0; code < ncell; code++) {
            int tx, ty, tz;
            morton_decode((uint32_t)code, tx, ty, tz);
            int s = (int)(code & 7);
            int ax = tx >> 1, ay = ty >> 1, az = tz >> 1;
            // M2L
            buf.clear();
            for (const StencilEntry& e : st.m2l[lt][s]) {
                int lev = e.mode == 1 ? k - 1 : k;
                int n = e.mode == 1 ? nk1 : nk;
                int vx = (e.mode == 1 ? ax : tx) + e.d[0];
                int vy = (e.mode == 1 ? ay : ty) + e.d[1];
                int vz = (e.mode == 1 ? az : tz) + e.d[2];
                int px = floordiv(vx, n), py = floordiv(vy, n), pz = floordiv(vz, n);
                if (!periodic && (px || py || pz)) continue;
                int ix = vx - px * n, iy = vy - py * n, iz = vz - pz * n;
                long key;
                if (e.mode == 1) {
                    key = ((long)pidx(px, py, pz) * (1L << (3 * (k - 1))) + morton_encode(ix, iy, iz)) * 9;
                } else {
                    int ob = ((ix & 1) << 2) | ((iy & 1) << 1) | (iz & 1);
                    key = ((long)pidx(px, py, pz) * (1L << (3 * (k - 1))) + morton_encode(ix >> 1, iy >> 1, iz >> 1)) * 9 +
                          1 + ob;
                }
                buf.push_back(E{key, (int)(level_base(lev) + morton_encode(ix, iy, iz)), px, py, pz});
            }
            std::sort(buf.begin(), buf.end(), [](const E& a, const E& b) { return a.key < b.key; });
            for (const E& x : buf) {
                m2l.tgt.push_back((int)(level_base(k) + code));
                m2l.src.push_back(x.src);
                m2l.off.push_back(x.ox);
                m2l.off.push_back(x.oy);
                m2l.off.push_back(x.oz);
            }
        }
    }
    // P2P at the leaf level
    {
        const int nD = 1 << D;
        const long ncell = 1L << (3 * D);
        for (long code = 0; code < ncell; code++) {
            int tx, ty, tz;
            morton_decode((uint32_t)code, tx, ty, tz);
            buf.clear();
            for (size_t i = 0; i < st.p2p.size() / 3; i++) {
                int vx = tx + st.p2p[3 * i], vy = ty + st.p2p[3 * i + 1], vz = tz + st.p2p[3 * i + 2];
                int px = floordiv(vx, nD), py = floordiv(vy, nD), pz = floordiv(vz, nD);
                if (!periodic && (px || py || pz)) continue;
                int ix = vx - px * nD, iy = vy - py * nD, iz = vz - pz * nD;
                long key = (long)pidx(px, py, pz) * ncell + morton_encode(ix, iy, iz);
                buf.push_back(E{key, (int)(level_base(D) + morton_encode(ix, iy, iz)), px, py, pz});
            }
            std::sort(buf.begin(), buf.end(), [](const E& a, const E& b) { return a.key < b.key; });
            for (const E& x : buf) {
                p2p.tgt.push_back((int)(level_base(D) + code));
                p2p.src.push_back(x.src);
                p2p.off.push_back(x.ox);
                p2p.off.push_back(x.oy);
                p2p.off.push_back(x.oz);
            }
        }
    }
}

}  // namespace gbfmm

// ------------------------------------------------------------------ tensor-core M2L plan

#include "m2l_tc.h"

namespace gbfmm {

static inline int round16(int x) { return (x + 15) & ~15; }

// Degree chunks by dynamic programming over contiguous degree ranges j0..j1
// (N = rows padded to 16, <= 256; K = (P-j0+1)^2 padded to 16).  The cost of a
// chunk per entry and product is its MMA issue, about 128 cycles per tcgen05.mma
// (M = 128, K = 16) whatever N is, plus the copy of its operator image (N rows of
// 128-byte K atoms at about 64 B/cycle).  The operator is zero where j + n > P
// (m2l_matrix), so a chunk may span more degrees than the truncation needs: at
// low orders one chunk is cheapest.  Where the images would keep two pipeline
// stages of the split-precision form from fitting a CTA's shared memory, the image
// bytes weigh more (make_tc_plan); the plan of fewest multiply-adds is the last
// resort.
static TcPlan tc_plan_dp(int P, int byte_weight)  // byte_weight 0: fewest multiply-adds
{
    TcPlan pl;
    pl.P = P;
    const int INF = 1 << 30;
    std::vector<int> best(P + 2, INF), nxt(P + 2, -1);
    best[P + 1] = 0;
    for (int j0 = P; j0 >= 0; j0--) {
        for (int j1 = j0; j1 <= P; j1++) {
            int rows = (j1 + 1) * (j1 + 1) - j0 * j0;
            int N = round16(rows);
            if (N > 256) break;
            int K = round16((P - j0 + 1) * (P - j0 + 1));
            int cost = byte_weight ? (K / 16) * 128 + N * ((K + 63) / 64) * byte_weight : N * K + 256;
            if (best[j1 + 1] < INF && cost + best[j1 + 1] < best[j0]) {
                best[j0] = cost + best[j1 + 1];
                nxt[j0] = j1 + 1;
            }
        }
    }
    int j0 = 0, col = 0, img = 0;
    while (j0 <= P) {
        int j1 = nxt[j0] - 1;
        int c = pl.nchunk++;
        pl.row0[c] = j0 * j0;
        pl.rows[c] = (j1 + 1) * (j1 + 1) - j0 * j0;
        pl.n[c] = round16(pl.rows[c]);
        pl.k[c] = round16((P - j0 + 1) * (P - j0 + 1));
        pl.col[c] = col;
        pl.img[c] = img;
        col += pl.n[c];
        img += pl.n[c] * ((pl.k[c] + 63) / 64) * 128;
        j0 = j1 + 1;
    }
    pl.img_bytes = img;
    pl.k_atoms = (pl.k[0] + 63) / 64;
    int t = 32;
    while (t < col) t <<= 1;
    pl.tmem_cols = t;
    return pl;
}

TcPlan make_tc_plan(int P)
{
    // two stages of hi and lo tiles (A: 128 rows per K atom, B: the images) within
    // 220 KB of shared memory (the kernel's static entry list and barriers take
    // the rest of the 227 KB): the image bytes weigh more until they fit
    for (int w = 2; w <= 64; w *= 2) {
        TcPlan pl = tc_plan_dp(P, w);
        const size_t stage = 2 * ((size_t)128 * pl.k_atoms * 128 + (size_t)pl.img_bytes);
        if (2 * stage <= 220 * 1024) return pl;
    }
    return tc_plan_dp(P, 0);
}

static uint16_t f2bf(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

static float bf2f(uint16_t b)
{
    uint32_t u = (uint32_t)b << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// Operator chunk images in the canonical K-major 128-byte-swizzled shared-memory
// layout: 64-element K atoms of N rows x 128 B; inside each 8-row group the
// 16-byte column chunk c of row r sits at chunk position c ^ (r & 7).
void append_tc_image(const TcPlan& pl, int R, const double* A, std::vector<uint8_t>& out)
{
    size_t base = out.size();
    out.resize(base + 2 * (size_t)pl.img_bytes, 0);
    for (int c = 0; c < pl.nchunk; c++) {
        const int N = pl.n[c], atoms = (pl.k[c] + 63) / 64;
        for (int nl = 0; nl < N; nl++) {
            const int r = pl.row0[c] + nl;
            for (int k = 0; k < atoms * 64; k++) {
                double x = (nl < pl.rows[c] && k < pl.k[c] && k < R) ? A[(size_t)r * R + k] : 0.0;
                uint16_t hi = f2bf((float)x);
                uint16_t lo = f2bf((float)(x - (double)bf2f(hi)));
                const int a = k / 64, kk = k % 64;
                size_t off = (size_t)pl.img[c] + (size_t)a * N * 128 + (size_t)nl * 128 +
                             (size_t)(((kk / 8) ^ (nl % 8)) * 16) + (size_t)(kk % 8) * 2;
                std::memcpy(&out[base + off], &hi, 2);
                std::memcpy(&out[base + pl.img_bytes + off], &lo, 2);
            }
        }
    }
}

}  // namespace gbfmm
