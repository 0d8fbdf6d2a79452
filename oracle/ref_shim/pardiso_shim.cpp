// Stand-in for the reference's MKL PARDISO wrapper (Code/OutputNu/pardiso.h,
// struct pardiso_solver), so that its smoothing classes (OutputResultant3d,
// Subdomain) build and run without MKL.  Only the symmetric real path that
// the smoothing uses does work: factorize_rsf keeps the matrix (lower
// triangle in the reference's row-sparse format: ig/jg/ggl plus the
// diagonal di, Subdomain.cpp:622) and solve_nrhs solves it by Jacobi-
// preconditioned conjugate gradients to a relative residual of 1e-15 (the
// matrices are nodal mass matrices, condition number below ~30 after
// diagonal scaling, so this is the direct solve's answer to rounding).
//
// Test infrastructure only (oracle/build_ref.sh, ref_smoothing).  Written
// for this repository; the reference's own pardiso.cpp (MKL calls) is not
// compiled.
#include "stdafx.h"
#include "pardiso.h"

#include <cmath>
#include <cstdlib>
#include <vector>

namespace {
struct Sym {
    int n = 0;
    std::vector<int> ig, jg;
    std::vector<double> gg, di;
    void mul(const double *x, double *y) const
    {
        for (int i = 0; i < n; i++) y[i] = di[i] * x[i];
        for (int i = 0; i < n; i++)
            for (int k = ig[i]; k < ig[i + 1]; k++) {
                const int j = jg[k];
                y[i] += gg[k] * x[j];
                y[j] += gg[k] * x[i];
            }
    }
};
}  // namespace

// the kept matrix hangs off the handle array that MKL would own (pt[0])
pardiso_solver::pardiso_solver()
{
    ia = nullptr;
    ja = nullptr;
    a = nullptr;
    perm = nullptr;
    n = 0;
    for (int i = 0; i < 64; i++) pt[i] = nullptr;
}

pardiso_solver::~pardiso_solver() { clear(); }

void pardiso_solver::init() {}
void pardiso_solver::init_rsf() {}

void pardiso_solver::clear()
{
    delete static_cast<Sym *>(pt[0]);
    pt[0] = nullptr;
    n = 0;
}

void pardiso_solver::stop_solver() { clear(); }

void pardiso_solver::factorize(int, int *, int *, double *, double *, double *, int *, int *, int)
{
    fprintf(stderr, "pardiso_shim: the non-symmetric factorisation is not provided\n");
    exit(70);
}

void pardiso_solver::factorize_rsf(int nb, int *ig, int *jg, double *ggl, double *di, int)
{
    clear();
    Sym *s = new Sym();
    s->n = nb;
    s->ig.assign(ig, ig + nb + 1);
    s->jg.assign(jg, jg + ig[nb]);
    s->gg.assign(ggl, ggl + ig[nb]);
    s->di.assign(di, di + nb);
    pt[0] = s;
    n = nb;
}

void pardiso_solver::solve_nrhs(int nrhs, double *pr, double *x)
{
    const Sym *s = static_cast<const Sym *>(pt[0]);
    if (!s) {
        fprintf(stderr, "pardiso_shim: solve before factorisation\n");
        exit(71);
    }
    const int N = s->n;
    std::vector<double> r(N), z(N), p(N), q(N);
    for (int c = 0; c < nrhs; c++) {
        const double *b = pr + (size_t)c * N;
        double *u = x + (size_t)c * N;
        s->mul(u, q.data());
        double bb = 0.0, rz = 0.0;
        for (int i = 0; i < N; i++) {
            r[i] = b[i] - q[i];
            z[i] = r[i] / s->di[i];
            p[i] = z[i];
            bb += b[i] * b[i];
            rz += r[i] * z[i];
        }
        const double tol2 = 1e-30 * bb;
        for (int it = 0; it < 10 * N + 100; it++) {
            double rr = 0.0;
            for (int i = 0; i < N; i++) rr += r[i] * r[i];
            if (rr <= tol2) break;
            s->mul(p.data(), q.data());
            double pq = 0.0;
            for (int i = 0; i < N; i++) pq += p[i] * q[i];
            if (pq <= 0.0) break;
            const double al = rz / pq;
            double rz2 = 0.0;
            for (int i = 0; i < N; i++) {
                u[i] += al * p[i];
                r[i] -= al * q[i];
                z[i] = r[i] / s->di[i];
                rz2 += r[i] * z[i];
            }
            const double be = rz2 / rz;
            rz = rz2;
            for (int i = 0; i < N; i++) p[i] = z[i] + be * p[i];
        }
    }
}
