// Host driver of the reference's own CPU FMM (TEST INFRASTRUCTURE ONLY): the
// kernel-independent FMM of src/gromacs/rtfmm, compiled unmodified from the
// reference checkout by oracle/rtfmm_build.sh (its tree depth, the literal 3 of
// fmm.cpp:21, read from rtfmm_depth() instead).  The calls follow
// rtFmmSolver::execute (src/gromacs/rtfmm/rtfmm_solver.cpp:14-56): Argument with
// its defaults, then P, n, images, the period box[XX][XX], the root half-width
// and centre; LaplaceFMM::solve; potentials and forces scaled by the Coulomb
// constant as the plugin does.
#include <cstdio>

#include "argument.h"
#include "fmm.h"

static int g_depth = 3;
extern "C" int rtfmm_depth() { return g_depth; }

extern "C" int rtfmm_ref_solve(int n, const double* xyz, const double* q, double L, int P, int depth, int images,
                               double* pot, double* force)
{
    if (n <= 0 || P < 2 || depth < 1 || depth > 6) return -1;
    g_depth = depth;
    char a0[] = "rtfmm";
    char* argv[] = {a0, nullptr};
    rtfmm::Argument args(1, argv);
    args.P = P;
    args.n = n;
    args.images = images;
    args.cycle = L;
    args.r = L / 2;
    args.x = rtfmm::vec3r(L / 2, L / 2, L / 2);
    args.timing = 0;
    rtfmm::Bodies3 bs(n);
    for (int i = 0; i < n; i++) {
        bs[i].idx = i;
        bs[i].p = 0;
        bs[i].f = rtfmm::vec3r(0, 0, 0);
        for (int m = 0; m < 3; m++) bs[i].x[m] = xyz[3 * i + m];
        bs[i].q = q[i];
    }
    rtfmm::LaplaceFMM fmm(bs, args);
    bs = fmm.solve();
    const double ke = 138.935457833;  // gmx::c_one4PiEps0, as rtfmm_solver.cpp:50-54 applies it
    for (int i = 0; i < n; i++) {
        pot[i] = bs[i].p * ke;
        for (int m = 0; m < 3; m++) force[3 * i + m] = -bs[i].q * bs[i].f[m] * ke;
    }
    return 0;
}
