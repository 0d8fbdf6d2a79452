/*
 * CPU oracle for the MTCalc solve stage — TEST INFRASTRUCTURE ONLY.
 * See mtcalc_oracle.h.  Restates, in plain C, the reference algorithms cited
 * at each function; reference paths are relative to the reference repo.
 * Only tests/, smoke() and bench.py's CPU-baseline arm use this file.
 */
#include "mtcalc_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

/* ------------------------------------------------------------------ helpers */
static double wall_seconds(void) { return omp_get_wtime(); }

static int clamp_threads(int t) { return t < 1 ? 1 : t; }

/* sum x_i^2, Code/COCR_FP/base_solver.cpp:41-69 (Scal, Norm_Euclid) */
static double norm2(const double *x, int n, int nt)
{
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) num_threads(nt) schedule(static)
    for (int i = 0; i < n; i++) s += x[i] * x[i];
    return s > 0.0 ? sqrt(s) : 0.0;
}

/* unconjugated complex dot, base_solver.cpp:382-399 (ScalCmplx) */
static double complex cdot(const double *x, const double *y, int nb, int nt)
{
    double sr = 0.0, si = 0.0;
#pragma omp parallel for reduction(+ : sr, si) num_threads(nt) schedule(static)
    for (int i = 0; i < nb; i++) {
        sr += x[2 * i] * y[2 * i] - x[2 * i + 1] * y[2 * i + 1];
        si += x[2 * i] * y[2 * i + 1] + x[2 * i + 1] * y[2 * i];
    }
    return sr + I * si;
}

/* z = x + a*y, base_solver.cpp:433-452 (Cmplx_axpy) */
static void caxpy(double complex a, const double *x, const double *y, double *z,
                  int nb, int nt)
{
    const double ar = creal(a), ai = cimag(a);
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int i = 0; i < nb; i++) {
        double tr = x[2 * i] + (y[2 * i] * ar - y[2 * i + 1] * ai);
        double ti = x[2 * i + 1] + (y[2 * i] * ai + y[2 * i + 1] * ar);
        z[2 * i] = tr;
        z[2 * i + 1] = ti;
    }
}

/* one 1- or 2-double block times a complex value, block_2x2_solver.cpp:41-53 */
static inline void block_mult(const double *a, int size, const double *x, double *y)
{
    if (size == 2) {
        y[0] += a[0] * x[0] - a[1] * x[1];
        y[1] += a[1] * x[0] + a[0] * x[1];
    } else {
        y[0] += a[0] * x[0];
        y[1] += a[0] * x[1];
    }
}

/* ------------------------------------------------------------------- SpMV */
/* Code/COCR_FP/block_2x2_solver.cpp:73-173.  With several threads each
 * thread scatters into its own buffer (thread 0 into y) and the buffers are
 * summed at the end, as the reference's y_omp scheme does. */
void orc_spmv_block2x2(int nb, const int *ig, const int *jg, const int *idi,
                       const int *ijg, const double *di, const double *gg,
                       const double *x, double *y, int nthreads)
{
    const int nt = clamp_threads(nthreads);
    const size_t n = (size_t)nb * 2;
    if (nt == 1) {
        memset(y, 0, n * sizeof(double));
        for (int i = 0; i < nb; i++) {
            block_mult(&di[idi[i]], idi[i + 1] - idi[i], &x[2 * i], &y[2 * i]);
            for (int j = ig[i]; j < ig[i + 1]; j++) {
                const int jb = 2 * jg[j];
                const int k = ijg[j], size = ijg[j + 1] - k;
                block_mult(&gg[k], size, &x[jb], &y[2 * i]);
                block_mult(&gg[k], size, &x[2 * i], &y[jb]);
            }
        }
        return;
    }
    double *extra = (double *)calloc(n * (size_t)(nt - 1), sizeof(double));
#pragma omp parallel num_threads(nt)
    {
        const int rank = omp_get_thread_num();
        double *dst = rank == 0 ? y : extra + (size_t)(rank - 1) * n;
        if (rank == 0) memset(y, 0, n * sizeof(double));
#pragma omp barrier
#pragma omp for schedule(static)
        for (int i = 0; i < nb; i++) {
            block_mult(&di[idi[i]], idi[i + 1] - idi[i], &x[2 * i], &dst[2 * i]);
            for (int j = ig[i]; j < ig[i + 1]; j++) {
                const int jb = 2 * jg[j];
                const int k = ijg[j], size = ijg[j + 1] - k;
                block_mult(&gg[k], size, &x[jb], &dst[2 * i]);
                block_mult(&gg[k], size, &x[2 * i], &dst[jb]);
            }
        }
#pragma omp for schedule(static)
        for (size_t i = 0; i < n; i++)
            for (int t = 0; t < nt - 1; t++) y[i] += extra[(size_t)t * n + i];
    }
    free(extra);
}

/* ------------------------------------------------- folded preconditioner */
/* Discrete gradient on the interior nodes of conductive cells:
 * Code/COCR_FP/FoldedPreconditioner.cpp:68-259 (BuildGMatrix).  Row e of G^T
 * holds -1/2 for the edge's first node and +1/2 for its second node (through
 * the T-matrix rows for non-conforming nodes). */
int orc_folded_build_g(orc_folded *p, int kpar, int n_edges_c, int n_nodes_c,
                       const int *nvkat, const int *nver14, const double *sigma3d,
                       const int *edges2, const int *ig_t, const int *jg_t,
                       const double *gg_t, const int *is_node_bound)
{
    memset(p, 0, sizeof(*p));
    p->n = n_edges_c;
    char *in_sigma = (char *)calloc((size_t)n_nodes_c + 1, 1);
    for (int c = 0; c < kpar; c++) {
        if (!(sigma3d[nvkat[c]] > 0.0)) continue;
        for (int j = 0; j < 8; j++) {
            int v = nver14[(size_t)c * 14 + j];
            if (v < n_nodes_c && !is_node_bound[v]) in_sigma[v] = 1;
        }
    }
    int *renum = (int *)malloc(sizeof(int) * (size_t)(n_nodes_c + 1));
    int m = 0;
    for (int v = 0; v < n_nodes_c; v++) renum[v] = in_sigma[v] ? m++ : -1;
    p->m = m;

    int *iptr = (int *)malloc(sizeof(int) * (size_t)(n_edges_c + 1));
    iptr[0] = 0;
    for (int e = 0; e < n_edges_c; e++) {
        int cnt = 0;
        for (int k = 0; k < 2; k++) {
            int v = edges2[2 * e + k];
            if (v < n_nodes_c) cnt += in_sigma[v];
            else
                for (int t = ig_t[v]; t < ig_t[v + 1]; t++) cnt += in_sigma[jg_t[t]];
        }
        iptr[e + 1] = iptr[e] + cnt;
    }
    const int nnz = iptr[n_edges_c];
    int *jptr = (int *)malloc(sizeof(int) * (size_t)(nnz + 1));
    double *val = (double *)malloc(sizeof(double) * (size_t)(nnz + 1));
    int w = 0;
    for (int e = 0; e < n_edges_c; e++)
        for (int k = 0; k < 2; k++) {
            int v = edges2[2 * e + k];
            const double sgn = k == 0 ? -0.5 : 0.5;
            if (v < n_nodes_c) {
                if (in_sigma[v]) { jptr[w] = renum[v]; val[w] = sgn; w++; }
            } else {
                for (int t = ig_t[v]; t < ig_t[v + 1]; t++)
                    if (in_sigma[jg_t[t]]) {
                        jptr[w] = renum[jg_t[t]];
                        val[w] = sgn * gg_t[t];
                        w++;
                    }
            }
        }
    /* transpose G^T -> G, rows of G list edges in increasing order */
    int *gp = (int *)calloc((size_t)m + 1, sizeof(int));
    for (int t = 0; t < nnz; t++) gp[jptr[t] + 1]++;
    for (int i = 0; i < m; i++) gp[i + 1] += gp[i];
    int *gj = (int *)malloc(sizeof(int) * (size_t)(nnz + 1));
    double *gv = (double *)malloc(sizeof(double) * (size_t)(nnz + 1));
    int *fill = (int *)malloc(sizeof(int) * (size_t)(m + 1));
    memcpy(fill, gp, sizeof(int) * (size_t)m);
    for (int e = 0; e < n_edges_c; e++)
        for (int t = iptr[e]; t < iptr[e + 1]; t++) {
            int r = jptr[t];
            gj[fill[r]] = e;
            gv[fill[r]] = val[t];
            fill[r]++;
        }
    free(fill);
    free(renum);
    free(in_sigma);
    p->iptr_gt = iptr; p->jptr_gt = jptr; p->gg_gt = val;
    p->iptr_g = gp; p->jptr_g = gj; p->gg_g = gv;
    return 0;
}

/* D_A = 1/diag(A) and D_S = 1/diag(G A G^T), both complex:
 * FoldedPreconditioner.cpp:473-574 (BuildDiagComplex) with the full block
 * rows of FoldedPreconditioner.cpp:633-737 (From2x2ToCSR2x2_*): lower part,
 * diagonal, then the mirrored upper part in increasing row order. */
int orc_folded_build_diag(orc_folded *p, const int *ig, const int *jg, const int *idi,
                          const int *ijg, const double *di, const double *gg)
{
    const int n = p->n, m = p->m;
    const int nnzl = ig[n];
    int *cnt = (int *)calloc((size_t)n + 1, sizeof(int));
    for (int i = 0; i < n; i++) {
        cnt[i] += ig[i + 1] - ig[i] + 1;
        for (int j = ig[i]; j < ig[i + 1]; j++) cnt[jg[j]]++;
    }
    int *fp = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    fp[0] = 0;
    for (int i = 0; i < n; i++) fp[i + 1] = fp[i] + cnt[i];
    const int nnzf = fp[n];
    int *fc = (int *)malloc(sizeof(int) * (size_t)nnzf);
    double *fv = (double *)malloc(sizeof(double) * 2 * (size_t)nnzf);
    for (int i = 0; i < n; i++) cnt[i] = fp[i];
    for (int i = 0; i < n; i++) {
        for (int j = ig[i]; j < ig[i + 1]; j++) {
            int q = cnt[i]++;
            fc[q] = jg[j];
            fv[2 * q] = gg[ijg[j]];
            fv[2 * q + 1] = (ijg[j + 1] - ijg[j] == 2) ? gg[ijg[j] + 1] : 0.0;
        }
        int q = cnt[i]++;
        fc[q] = i;
        fv[2 * q] = di[idi[i]];
        fv[2 * q + 1] = (idi[i + 1] - idi[i] == 2) ? di[idi[i] + 1] : 0.0;
    }
    for (int i = 0; i < n; i++)
        for (int j = ig[i]; j < ig[i + 1]; j++) {
            int k = jg[j];
            int q = cnt[k]++;
            fc[q] = i;
            fv[2 * q] = gg[ijg[j]];
            fv[2 * q + 1] = (ijg[j + 1] - ijg[j] == 2) ? gg[ijg[j] + 1] : 0.0;
        }
    (void)nnzl;

    p->diag_a = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    for (int i = 0; i < n; i++) {
        double complex a = di[idi[i]] + I * ((idi[i + 1] - idi[i] == 2) ? di[idi[i] + 1] : 0.0);
        double complex r = 1.0 / a;
        p->diag_a[2 * i] = creal(r);
        p->diag_a[2 * i + 1] = cimag(r);
    }
    p->diag_gagt = (double *)calloc(2 * (size_t)m + 2, sizeof(double));
    p->help = (double *)calloc(2 * (size_t)m + 2, sizeof(double));
    for (int i = 0; i < m; i++) {
        for (int j = p->iptr_g[i]; j < p->iptr_g[i + 1]; j++) {
            const int k = p->jptr_g[j];
            double sr = 0.0, si = 0.0;
            for (int q = fp[k]; q < fp[k + 1]; q++) {
                const int c = fc[q];
                for (int t = p->iptr_g[i]; t < p->iptr_g[i + 1]; t++)
                    if (p->jptr_g[t] == c) {
                        sr += fv[2 * q] * p->gg_g[t];
                        si += fv[2 * q + 1] * p->gg_g[t];
                    }
            }
            p->diag_gagt[2 * i] += sr * p->gg_g[j];
            p->diag_gagt[2 * i + 1] += si * p->gg_g[j];
        }
    }
    for (int i = 0; i < m; i++) {
        double complex r = 1.0 / (p->diag_gagt[2 * i] + I * p->diag_gagt[2 * i + 1]);
        p->diag_gagt[2 * i] = creal(r);
        p->diag_gagt[2 * i + 1] = cimag(r);
    }
    free(cnt); free(fp); free(fc); free(fv);
    return 0;
}

/* y = D_A x + G^T D_S G x, FoldedPreconditioner.cpp:578-630. */
void orc_folded_apply(const orc_folded *p, const double *x, double *y, int nthreads)
{
    const int nt = clamp_threads(nthreads);
    const int n = p->n, m = p->m;
    double *h = p->help;
#pragma omp parallel num_threads(nt)
    {
#pragma omp for schedule(static) nowait
        for (int i = 0; i < n; i++) {
            const double ar = p->diag_a[2 * i], ai = p->diag_a[2 * i + 1];
            y[2 * i] = x[2 * i] * ar - x[2 * i + 1] * ai;
            y[2 * i + 1] = x[2 * i] * ai + x[2 * i + 1] * ar;
        }
#pragma omp for schedule(static)
        for (int i = 0; i < m; i++) {
            double hr = 0.0, hi = 0.0;
            for (int j = p->iptr_g[i]; j < p->iptr_g[i + 1]; j++) {
                const int k = p->jptr_g[j];
                hr += p->gg_g[j] * x[2 * k];
                hi += p->gg_g[j] * x[2 * k + 1];
            }
            const double dr = p->diag_gagt[2 * i], dim = p->diag_gagt[2 * i + 1];
            h[2 * i] = hr * dr - hi * dim;
            h[2 * i + 1] = hi * dr + hr * dim;
        }
#pragma omp for schedule(static)
        for (int i = 0; i < n; i++)
            for (int j = p->iptr_gt[i]; j < p->iptr_gt[i + 1]; j++) {
                const int k = p->jptr_gt[j];
                y[2 * i] += p->gg_gt[j] * h[2 * k];
                y[2 * i + 1] += p->gg_gt[j] * h[2 * k + 1];
            }
    }
}

void orc_folded_free(orc_folded *p)
{
    free(p->iptr_g); free(p->jptr_g); free(p->gg_g);
    free(p->iptr_gt); free(p->jptr_gt); free(p->gg_gt);
    free(p->diag_a); free(p->diag_gagt); free(p->help);
    memset(p, 0, sizeof(*p));
}

/* --------------------------------------------------------------- the solve */
/* Real-valued minimal residual smoothing of the residual, MRS.cpp:85-153.
 * Only the smoothed residual s (and its norm) is observable: the smoothed
 * iterate is never read back by the reference, so it is not kept here. */
typedef struct {
    double *s, *u;
    int n, init;
    double residual;
} mrs_state;

static void mrs_step(mrs_state *M, const double *r, int nt)
{
    const int n = M->n;
    if (!M->init) {
        memcpy(M->s, r, sizeof(double) * (size_t)n);
        M->residual = norm2(M->s, n, nt);
        M->init = 1;
        return;
    }
    double su = 0.0, uu = 0.0;
#pragma omp parallel for reduction(+ : su, uu) num_threads(nt) schedule(static)
    for (int i = 0; i < n; i++) {
        M->u[i] = r[i] - M->s[i];
        su += M->s[i] * M->u[i];
        uu += M->u[i] * M->u[i];
    }
    double w = fabs(uu) < 1e-100 ? 0.0 : -su / uu;
    if (w < 0.0) return;               /* w clamped to 0: s and the norm stay */
    if (w > 1.0) {                     /* w clamped to 1: restart from r */
        memcpy(M->s, r, sizeof(double) * (size_t)n);
        M->residual = norm2(M->s, n, nt);
        return;
    }
    double res = 0.0;
#pragma omp parallel for reduction(+ : res) num_threads(nt) schedule(static)
    for (int i = 0; i < n; i++) {
        M->s[i] += w * M->u[i];
        res += M->s[i] * M->s[i];
    }
    M->residual = sqrt(res);
}

/* PCOCR_2x2_Folded, pcocr.cpp:40-126, with the state machine of
 * PCOCR_RCI::Run (pcocr_rci.cpp:52-181) written as one loop.  `iter_limit`
 * (0 = none) stops after that many iterations and returns ORC_REQ_MAXITER;
 * the benchmark uses it to time a bounded sample of a long solve. */
int orc_pcocr_2x2_folded(int n, const int *ig, const int *jg, const int *idi,
                         const int *ijg, const double *di, const double *gg,
                         const double *pr, double *x, double eps, int maxiter,
                         int kpar, int n_edges_c, int n_nodes_c,
                         const int *nvkat, const int *nver14, const double *sigma3d,
                         const int *edges2, const int *ig_t, const int *jg_t,
                         const double *gg_t, const int *is_node_bound,
                         int nthreads, int iter_limit, orc_stats *st)
{
    const int nt = clamp_threads(nthreads);
    const int nb = n / 2;
    const double t0 = wall_seconds();
    double *r = (double *)malloc(sizeof(double) * (size_t)n);
    double *p = (double *)calloc((size_t)n, sizeof(double));
    double *s = (double *)malloc(sizeof(double) * (size_t)n);
    double *z = (double *)malloc(sizeof(double) * (size_t)n);
    double *a = (double *)calloc((size_t)n, sizeof(double));
    double *w = (double *)calloc((size_t)n, sizeof(double));
    mrs_state M = {(double *)malloc(sizeof(double) * (size_t)n),
                   (double *)malloc(sizeof(double) * (size_t)n), n, 0, -1.0};
    orc_folded P;
    orc_folded_build_g(&P, kpar, n_edges_c, n_nodes_c, nvkat, nver14, sigma3d, edges2,
                       ig_t, jg_t, gg_t, is_node_bound);
    orc_folded_build_diag(&P, ig, jg, idi, ijg, di, gg);

    int req = ORC_REQ_OK, iter = 0;
    double residual_rel = 1.0;
    double complex beta = 0.0, zs, zs_old, aw, alpha;

    orc_spmv_block2x2(nb, ig, jg, idi, ijg, di, gg, x, r, nt);        /* stage 1 */
    for (int i = 0; i < n; i++) r[i] = pr[i] - r[i];                    /* stage 2 */
    const double r_old = norm2(pr, n, nt);
    mrs_step(&M, r, nt);                                                /* x0 test */
    if (norm2(r, n, nt) < 1e-30) { req = ORC_REQ_X0_NULL; goto done; }
    orc_folded_apply(&P, r, s, nt);                                     /* stage 3 */
    orc_spmv_block2x2(nb, ig, jg, idi, ijg, di, gg, s, z, nt);        /* stage 4 */

    for (;;) {
        iter++;                                                         /* stage 5 */
        if (iter > maxiter || (iter_limit > 0 && iter > iter_limit)) {
            req = ORC_REQ_MAXITER;
            break;
        }
        caxpy(beta, s, p, p, nb, nt);
        caxpy(beta, z, a, a, nb, nt);
        zs = cdot(z, s, nb, nt);
        orc_folded_apply(&P, a, w, nt);
        aw = cdot(a, w, nb, nt);                                        /* stage 6 */
        if (fabs(creal(aw)) < 1e-40 && fabs(cimag(aw)) < 1e-40) {
            req = ORC_REQ_DIV_BY_ZERO;
            break;
        }
        alpha = zs / aw;
        caxpy(alpha, x, p, x, nb, nt);
        caxpy(-alpha, r, a, r, nb, nt);
        mrs_step(&M, r, nt);                                            /* stop test */
        residual_rel = M.residual / r_old;
        if (residual_rel < eps) { req = ORC_REQ_OK; break; }
        caxpy(-alpha, s, w, s, nb, nt);                                 /* stage 7 */
        orc_spmv_block2x2(nb, ig, jg, idi, ijg, di, gg, s, z, nt);
        zs_old = zs;                                                    /* stage 8 */
        zs = cdot(z, s, nb, nt);
        beta = zs / zs_old;
    }
done:
    if (st) {
        st->iterations = iter;
        st->residual_rel = residual_rel;
        st->seconds = wall_seconds() - t0;
    }
    orc_folded_free(&P);
    free(r); free(p); free(s); free(z); free(a); free(w); free(M.s); free(M.u);
    return req;
}

/* --------------------------------------------------------------- assembly */
static int cmp_u64(const void *a, const void *b)
{
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

/* Lower-triangular edge adjacency: Code/BuildMatrix/T_Portrait.cpp:47-124
 * (Gen_Portrait).  Row b lists, ascending, every edge a < b sharing a cell. */
int orc_portrait(int nb, int kpar, const int *ed12, int ed_stride, int *ig, int **jg_out)
{
    size_t cap = (size_t)kpar * 66, cnt = 0;
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (cap ? cap : 1));
    for (int c = 0; c < kpar; c++) {
        const int *e = ed12 + (size_t)c * ed_stride;
        for (int j = 0; j < 12; j++)
            for (int k = 0; k < 12; k++)
                if (e[k] < e[j]) keys[cnt++] = ((uint64_t)(uint32_t)e[j] << 32) | (uint32_t)e[k];
        if (cnt + 144 > cap) {
            cap *= 2;
            keys = (uint64_t *)realloc(keys, sizeof(uint64_t) * cap);
        }
    }
    qsort(keys, cnt, sizeof(uint64_t), cmp_u64);
    size_t u = 0;
    for (size_t i = 0; i < cnt; i++)
        if (u == 0 || keys[i] != keys[u - 1]) keys[u++] = keys[i];
    int *jg = (int *)malloc(sizeof(int) * (u ? u : 1));
    memset(ig, 0, sizeof(int) * (size_t)(nb + 1));
    for (size_t i = 0; i < u; i++) {
        ig[(keys[i] >> 32) + 1]++;
        jg[i] = (int)(keys[i] & 0xffffffffu);
    }
    for (int i = 0; i < nb; i++) ig[i + 1] += ig[i];
    free(keys);
    *jg_out = jg;
    return (int)u;
}

static int find_in_row(const int *ig, const int *jg, int row, int col)
{
    int lo = ig[row], hi = ig[row + 1] - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (jg[mid] == col) return mid;
        if (jg[mid] < col) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

/* Block sizes: 2 doubles (complex) for parallel edge pairs and every
 * diagonal, 1 double (real) for perpendicular pairs.
 * T_Portrait.cpp:126-188 with the direction filter of T_Portrait.h:37-51
 * (local edges 0-3, 4-7, 8-11 are the x, y, z groups). */
void orc_block_types(int nb, int kpar, const int *ed12, int ed_stride,
                     const int *ig, const int *jg, int *idi, int *ijg)
{
    const int nnz = ig[nb];
    for (int i = 0; i <= nb; i++) idi[i] = 2;
    for (int i = 0; i <= nnz; i++) ijg[i] = 1;
    for (int c = 0; c < kpar; c++) {
        const int *e = ed12 + (size_t)c * ed_stride;
        for (int j = 0; j < 12; j++)
            for (int k = 0; k < 12; k++)
                if (e[k] < e[j] && j / 4 == k / 4) {
                    int q = find_in_row(ig, jg, e[j], e[k]);
                    if (q >= 0) ijg[q] = 2;
                }
    }
    /* sizes -> offsets */
    int acc = 0;
    for (int i = 0; i < nb; i++) { int t = idi[i]; idi[i] = acc; acc += t; }
    idi[nb] = acc;
    acc = 0;
    for (int i = 0; i < nnz; i++) { int t = ijg[i]; ijg[i] = acc; acc += t; }
    ijg[nnz] = acc;
}

/* Local 12x12 curl-curl (b) and mass (c) matrices of an axis-aligned brick,
 * equal to the closed forms of T_Brick.cpp:123-455.  Written here from the
 * tensor-product structure of the lowest-order edge basis: with the 1-D
 * reference mass weights M(same)=2/3, M(diff)=1/3 and stiffness signs
 * K(same)=+1, K(diff)=-1,
 *   same direction d, transverse axes t1, t2:
 *     b = m[t1] K(t2) M(t1) + m[t2] K(t1) M(t2),  m[t] = 2 h_t / (h_d h_o)
 *     c = (h_t1 h_t2 / h_d) M(t1) M(t2)
 *   directions d_a != d_b, third axis q:
 *     b = -(2 h_q / (h_da h_db)) s(pos_a[d_b]) s(pos_b[d_a]) M(q),  s(0)=-1, s(1)=+1
 *     c = 0
 * where pos[e][axis] is the edge's side (0/1) along a transverse axis. */
static const signed char LOCAL_DIR[12] = {0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2};
/* side along x, y, z of each local edge (-1 along its own direction),
 * from the edge midpoints of T_Brick.h:201-214 */
static const signed char LOCAL_POS[12][3] = {
    {-1, 0, 0}, {-1, 1, 0}, {-1, 0, 1}, {-1, 1, 1},
    {0, -1, 0}, {0, -1, 1}, {1, -1, 0}, {1, -1, 1},
    {0, 0, -1}, {1, 0, -1}, {0, 1, -1}, {1, 1, -1}};

void orc_brick_bc(double hx, double hy, double hz, double *b, double *c)
{
    const double h[3] = {hx, hy, hz};
    for (int i = 0; i < 12; i++)
        for (int j = 0; j < 12; j++) {
            const int da = LOCAL_DIR[i], db = LOCAL_DIR[j];
            double bv, cv = 0.0;
            if (da == db) {
                const int t1 = (da + 1) % 3, t2 = (da + 2) % 3;
                const int s1 = LOCAL_POS[i][t1] == LOCAL_POS[j][t1];
                const int s2 = LOCAL_POS[i][t2] == LOCAL_POS[j][t2];
                const double M1 = s1 ? 2.0 / 3.0 : 1.0 / 3.0, M2 = s2 ? 2.0 / 3.0 : 1.0 / 3.0;
                const double K1 = s1 ? 1.0 : -1.0, K2 = s2 ? 1.0 : -1.0;
                const double m1 = 2.0 * h[t1] / (h[da] * h[t2]);
                const double m2 = 2.0 * h[t2] / (h[da] * h[t1]);
                bv = m1 * K2 * M1 + m2 * K1 * M2;
                cv = (h[t1] * h[t2] / h[da]) * M1 * M2;
            } else {
                const int q = 3 - da - db;
                const double sa = LOCAL_POS[i][db] ? 1.0 : -1.0;
                const double sb = LOCAL_POS[j][da] ? 1.0 : -1.0;
                const double Mq = LOCAL_POS[i][q] == LOCAL_POS[j][q] ? 2.0 / 3.0 : 1.0 / 3.0;
                bv = -(2.0 * h[q] / (h[da] * h[db])) * sa * sb * Mq;
            }
            b[i * 12 + j] = bv;
            c[i * 12 + j] = cv;
        }
}

/* Code/BuildMatrix/For_Solvers.cpp:236-270 (Spline): linear interpolation,
 * constant beyond the table ends. */
double orc_spline(double x, int n, const double *z, const double *v)
{
    if (x < z[0]) return v[0];
    if (x > z[n - 1]) return v[n - 1];
    for (int i = 0; i < n - 1; i++)
        if (x >= z[i] && x <= z[i + 1]) {
            const double xi = (x - z[i]) / (z[i + 1] - z[i]);
            return (1.0 - xi) * v[i] + xi * v[i + 1];
        }
    return 0.0;
}

/* Global assembly: Code/BuildMatrix/t_global_slae.cpp:80-172 (AsmBlockSLAE,
 * Add_to_*), local terms T_Brick.cpp:1361-1395 and 1463-1495, boundary
 * conditions bound_cond_vec_harm.cpp:81-108 and 260-307. */
int orc_assemble(int nb, int kpar, const double *xyz, const int *nver14,
                 const int *ed12, int ed_stride, const int *edges2,
                 const int *nvkat, const double *mu3d, const double *mu0,
                 const double *sigma3d, const double *sigma0,
                 const double *dpr3d, const double *dpr0,
                 double nu, int alfa, int n1d, const double *z1d,
                 const double *usin, const double *ucos,
                 int kuzlov, int kt1, const int *l13d,
                 const int *ig, const int *jg, const int *idi, const int *ijg,
                 double *di, double *gg, double *pr)
{
    const double PI = 3.1415926535897932384626433832795;   /* BuildMatrix/stdafx.h:32 */
    const double omega = 2.0 * PI * nu;
    const int nnz = ig[nb];
    memset(di, 0, sizeof(double) * (size_t)idi[nb]);
    memset(gg, 0, sizeof(double) * (size_t)ijg[nnz]);
    memset(pr, 0, sizeof(double) * 2 * (size_t)nb);
    double b[144], c[144];
    for (int cell = 0; cell < kpar; cell++) {
        const int *nv = nver14 + (size_t)cell * 14;
        const int *e = ed12 + (size_t)cell * ed_stride;
        const int mat = nvkat[cell];
        const double hx = xyz[3 * nv[7] + 0] - xyz[3 * nv[0] + 0];
        const double hy = xyz[3 * nv[7] + 1] - xyz[3 * nv[0] + 1];
        const double hz = xyz[3 * nv[7] + 2] - xyz[3 * nv[0] + 2];
        const double h[3] = {hx, hy, hz};
        orc_brick_bc(hx, hy, hz, b, c);
        /* normal field at edge midpoints, dotted with J t = (h_d / 2) e_d */
        double as[12], ac[12];
        for (int i = 0; i < 12; i++) {
            const int n1 = edges2[2 * e[i]], n2 = edges2[2 * e[i] + 1];
            const double zm = 0.5 * (xyz[3 * n1 + 2] + xyz[3 * n2 + 2]);
            const int d = LOCAL_DIR[i];
            const double fs = orc_spline(zm, n1d, z1d, usin);
            const double fc = orc_spline(zm, n1d, z1d, ucos);
            const double w = d == 0 ? (double)alfa : (d == 1 ? 1.0 - (double)alfa : 0.0);
            as[i] = d == 2 ? 0.0 : 0.5 * h[d] * (fs * w);
            ac[i] = d == 2 ? 0.0 : 0.5 * h[d] * (fc * w);
        }
        double gre[12], gim[12], greb[12], gimb[12];
        for (int i = 0; i < 12; i++) {
            double s1 = 0, s2 = 0, s3 = 0, s4 = 0;
            for (int j = 0; j < 12; j++) {
                s1 += c[i * 12 + j] * as[j];
                s2 += c[i * 12 + j] * ac[j];
                s3 += b[i * 12 + j] * as[j];
                s4 += b[i * 12 + j] * ac[j];
            }
            gre[i] = s1; gim[i] = s2; greb[i] = s3; gimb[i] = s4;
        }
        const double mu = mu3d[mat], sig = sigma3d[mat], dpr = dpr3d[mat];
        const double mult = (sigma0[mat] - sig) * omega;
        const double mult_dpr = (dpr0[mat] - dpr) * omega * omega;
        const double mult_mu = 1.0 / mu0[mat] - 1.0 / mu;
        for (int i = 0; i < 144; i++) {
            b[i] = b[i] / mu - dpr * omega * omega * c[i];
            c[i] *= sig * omega;
        }
        for (int j = 0; j < 12; j++) {
            const int ii = e[j];
            di[idi[ii]] += b[j * 12 + j];
            if (idi[ii + 1] - idi[ii] == 2) di[idi[ii] + 1] += c[j * 12 + j];
            pr[2 * ii] += gim[j] * (-mult) - gre[j] * mult_dpr + greb[j] * mult_mu;
            pr[2 * ii + 1] += gre[j] * mult - gim[j] * mult_dpr + gimb[j] * mult_mu;
            for (int k = 0; k < 12; k++) {
                const int jj = e[k];
                if (jj >= ii) continue;
                const int q = find_in_row(ig, jg, ii, jj);
                if (q < 0) continue;
                gg[ijg[q]] += b[j * 12 + k];
                if (ijg[q + 1] - ijg[q] == 2) gg[ijg[q] + 1] += c[j * 12 + k];
            }
        }
    }
    /* homogeneous Dirichlet: an edge with both nodes on the boundary */
    char *nb_flag = (char *)calloc((size_t)kuzlov, 1);
    char *eb = (char *)calloc((size_t)nb, 1);
    for (int i = 0; i < kt1; i++) nb_flag[l13d[i]] = 1;
    for (int i = 0; i < nb; i++) eb[i] = nb_flag[edges2[2 * i]] && nb_flag[edges2[2 * i + 1]];
    for (int i = 0; i < nb; i++) {
        if (eb[i]) {
            di[idi[i]] = 1.0;
            if (idi[i + 1] - idi[i] == 2) di[idi[i] + 1] = 0.0;
            for (int j = ig[i]; j < ig[i + 1]; j++) {
                gg[ijg[j]] = 0.0;
                if (ijg[j + 1] - ijg[j] == 2) gg[ijg[j] + 1] = 0.0;
            }
            pr[2 * i] = pr[2 * i + 1] = 0.0;
        }
        for (int j = ig[i]; j < ig[i + 1]; j++)
            if (eb[jg[j]]) {
                gg[ijg[j]] = 0.0;
                if (ijg[j + 1] - ijg[j] == 2) gg[ijg[j] + 1] = 0.0;
            }
    }
    free(nb_flag);
    free(eb);
    return 0;
}

/* Test helper: build the folded preconditioner for an SLAE and apply it once;
 * returns m and copies 1/diag(A) and 1/diag(G A G^T) out. */
int orc_folded_apply_once(int nb, const int *ig, const int *jg, const int *idi, const int *ijg,
                          const double *di, const double *gg, int kpar, int n_nodes_c,
                          const int *nvkat, const int *nver14, const double *sigma3d,
                          const int *edges2, const int *ig_t, const int *jg_t,
                          const double *gg_t, const int *is_node_bound, const double *x,
                          double *y, double *diag_a, double *diag_gagt)
{
    orc_folded P;
    orc_folded_build_g(&P, kpar, nb, n_nodes_c, nvkat, nver14, sigma3d, edges2, ig_t, jg_t,
                       gg_t, is_node_bound);
    orc_folded_build_diag(&P, ig, jg, idi, ijg, di, gg);
    orc_folded_apply(&P, x, y, 1);
    memcpy(diag_a, P.diag_a, sizeof(double) * 2 * (size_t)nb);
    memcpy(diag_gagt, P.diag_gagt, sizeof(double) * 2 * (size_t)P.m);
    const int m = P.m;
    orc_folded_free(&P);
    return m;
}

/* ---- receivers and MT responses ------------------------------------------ */

/* Code/OutputNu/OutputArbitrary.cpp:385-500: the reference scans the elements
 * in index order and keeps, for every receiver, the first whose closed box
 * (vertex 0 to vertex 7, exact comparisons) holds it. */
int orc_locate_receivers(int kpar, const int *nver14, const double *xyz, int nrec,
                         const double *rec, int *elem)
{
    int missing = 0;
    for (int r = 0; r < nrec; r++) {
        const double *p = rec + 3 * r;
        elem[r] = -1;
        for (int e = 0; e < kpar; e++) {
            const double *lo = xyz + 3 * nver14[14 * e + 0];
            const double *hi = xyz + 3 * nver14[14 * e + 7];
            if (p[0] >= lo[0] && p[1] >= lo[1] && p[2] >= lo[2] &&
                p[0] <= hi[0] && p[1] <= hi[1] && p[2] <= hi[2]) {
                elem[r] = e;
                break;
            }
        }
        if (elem[r] < 0) missing++;
    }
    return missing;
}

static double lin0(double t) { return 0.5 * (1.0 - t); }
static double lin1(double t) { return 0.5 * (1.0 + t); }

/* Lowest-order edge basis on a brick with local coordinates in [-1,1]^3
 * (T_Brick.cpp:980-1060): edge i of direction d carries the tangential
 * component (2/h_d) l_a l_b in the two other local coordinates.  The curl
 * components follow from l0' = -1/2, l1' = +1/2 (T_Brick.cpp:1484-1618,
 * 1842-1918): each depends on one local coordinate only. */
void orc_receiver_eval(const int *nver14, const int *ed25, const double *xyz, int nrec,
                       const double *rec, const int *elem, const double *v3,
                       double *a, double *curl)
{
    for (int r = 0; r < nrec; r++) {
        double *ar = a + 6 * r, *cr = curl + 6 * r;
        for (int k = 0; k < 6; k++) ar[k] = cr[k] = 0.0;
        const int e = elem[r];
        if (e < 0) continue;
        const double *lo = xyz + 3 * nver14[14 * e + 0];
        const double *hi = xyz + 3 * nver14[14 * e + 7];
        const double hx = hi[0] - lo[0], hy = hi[1] - lo[1], hz = hi[2] - lo[2];
        const double *p = rec + 3 * r;
        const double xi = (2.0 * p[0] - lo[0] - hi[0]) / hx;
        const double et = (2.0 * p[1] - lo[1] - hi[1]) / hy;
        const double ze = (2.0 * p[2] - lo[2] - hi[2]) / hz;
        for (int part = 0; part < 2; part++) {
            double v[12];
            for (int i = 0; i < 12; i++) v[i] = v3[2 * ed25[25 * e + i] + part];
            ar[0 + part] = 2.0 / hx * (v[0] * lin0(et) * lin0(ze) + v[1] * lin1(et) * lin0(ze) +
                                       v[2] * lin0(et) * lin1(ze) + v[3] * lin1(et) * lin1(ze));
            ar[2 + part] = 2.0 / hy * (v[4] * lin0(ze) * lin0(xi) + v[5] * lin1(ze) * lin0(xi) +
                                       v[6] * lin0(ze) * lin1(xi) + v[7] * lin1(ze) * lin1(xi));
            ar[4 + part] = 2.0 / hz * (v[8] * lin0(xi) * lin0(et) + v[9] * lin1(xi) * lin0(et) +
                                       v[10] * lin0(xi) * lin1(et) + v[11] * lin1(xi) * lin1(et));
            /* curl_x = dAz/dy - dAy/dz, curl_y = dAx/dz - dAz/dx, curl_z = dAy/dx - dAx/dy */
            cr[0 + part] = 2.0 / (hy * hz) * (lin0(xi) * (v[4] - v[5] - v[8] + v[10]) +
                                              lin1(xi) * (v[6] - v[7] - v[9] + v[11]));
            cr[2 + part] = 2.0 / (hx * hz) * (lin0(et) * (v[2] - v[0] + v[8] - v[9]) +
                                              lin1(et) * (v[3] - v[1] + v[10] - v[11]));
            cr[4 + part] = 2.0 / (hx * hy) * (lin0(ze) * (v[0] - v[1] - v[4] + v[6]) +
                                              lin1(ze) * (v[2] - v[3] - v[5] + v[7]));
        }
    }
}

/* Code/Harm1D/divgrad_1d.cpp:90-138: outside [z1, z_{n-2}] the end slopes;
 * inside, the node slopes (weighted averages of the two adjacent slopes) at
 * the ends of the containing interval, interpolated linearly; where one of
 * them does not exist, the interval's own slope. */
double orc_dspline(double x, int n, const double *z, const double *v)
{
    if (x < z[1]) return (v[1] - v[0]) / (z[1] - z[0]);
    if (x > z[n - 2]) return (v[n - 1] - v[n - 2]) / (z[n - 1] - z[n - 2]);
    int i = 1;
    while (i < n && !(x <= z[i])) i++;
    double d0 = 0.0, d1 = 0.0;
    int f0 = 0, f1 = 0;
    if (i - 1 > 0) {
        f0 = 1;
        const double w = (z[i - 1] - z[i - 2]) / (z[i] - z[i - 2]);
        const double s0 = (v[i - 1] - v[i - 2]) / (z[i - 1] - z[i - 2]);
        const double s1 = (v[i] - v[i - 1]) / (z[i] - z[i - 1]);
        d0 = s0 * (1.0 - w) + s1 * w;
    }
    if (i + 1 < n) {
        f1 = 1;
        const double w = (z[i] - z[i - 1]) / (z[i + 1] - z[i - 1]);
        const double s0 = (v[i] - v[i - 1]) / (z[i] - z[i - 1]);
        const double s1 = (v[i + 1] - v[i]) / (z[i + 1] - z[i]);
        d1 = s0 * (1.0 - w) + s1 * w;
    }
    if (f0 && f1) {
        const double t = (x - z[i - 1]) / (z[i] - z[i - 1]);
        return (1.0 - t) * d0 + t * d1;
    }
    return (v[i] - v[i - 1]) / (z[i] - z[i - 1]);   /* one node slope missing: the interval's */
}

/* Code/Harm1D/divgrad_1d.cpp:290-330.  b: below the surface the z-derivative
 * of the 1-D potential, above it the air value B = MU0 (unit H); e: the
 * potential itself, taken at z = 0 for receivers above the surface. */
void orc_normal_field(double z, int n1d, const double *z1d, const double *usin,
                      const double *ucos, int alfa, double omega, double *e, double *b)
{
    const double mu = 4.0 * 3.1415926535897932 * 1e-7;   /* Code/Harm1D/divgrad_1d.cpp:288 */
    const double a = (double)alfa;
    double ds, dc;
    if (z < 0.0) {
        ds = orc_dspline(z, n1d, z1d, usin);
        dc = orc_dspline(z, n1d, z1d, ucos);
    } else {
        ds = mu;
        dc = 0.0;
    }
    b[0] = (a - 1.0) * ds; b[1] = a * ds; b[2] = 0.0;
    b[3] = (a - 1.0) * dc; b[4] = a * dc; b[5] = 0.0;
    const double zz = (z > 0.0) ? 0.0 : z;
    const double us = orc_spline(zz, n1d, z1d, usin);
    const double uc = orc_spline(zz, n1d, z1d, ucos);
    e[0] = omega * a * uc;  e[1] = omega * (1.0 - a) * uc; e[2] = 0.0;
    e[3] = -omega * a * us; e[4] = omega * (a - 1.0) * us; e[5] = 0.0;
}

#define ORC_MU0 1.25663706143591729e-6   /* Code/OutputNu/stdafx.h:31 */

void orc_receiver_fields(int nrec, const double *a, const double *curl, double omega,
                         const double *e1d, const double *b1d, double *e, double *h,
                         double *rho_imp)
{
    for (int r = 0; r < nrec; r++) {
        const double *ar = a + 6 * r, *cr = curl + 6 * r;
        double *er = e + 6 * r, *hr = h + 6 * r;
        for (int d = 0; d < 3; d++) {
            /* E = -i omega A (give_out_vec_mt.cpp:141-165), H = curl A / mu0 (:173-195) */
            er[2 * d] = omega * ar[2 * d + 1];
            er[2 * d + 1] = -omega * ar[2 * d];
            hr[2 * d] = cr[2 * d] / ORC_MU0;
            hr[2 * d + 1] = cr[2 * d + 1] / ORC_MU0;
        }
        /* normal field on x and y (give_out_vec_mt.cpp:58-99, 239-245) */
        for (int d = 0; d < 2; d++) {
            er[2 * d] += e1d[6 * r + d];
            er[2 * d + 1] += e1d[6 * r + 3 + d];
            hr[2 * d] += b1d[6 * r + d] / ORC_MU0;
            hr[2 * d + 1] += b1d[6 * r + 3 + d] / ORC_MU0;
        }
        /* give_out_vec_mt.cpp:247-264: moduli of the real and imaginary parts */
        const double ere = sqrt(er[0] * er[0] + er[2] * er[2] + er[4] * er[4]);
        const double eim = sqrt(er[1] * er[1] + er[3] * er[3] + er[5] * er[5]);
        const double hre = sqrt(hr[0] * hr[0] + hr[2] * hr[2] + hr[4] * hr[4]);
        const double him = sqrt(hr[1] * hr[1] + hr[3] * hr[3] + hr[5] * hr[5]);
        const double ea = sqrt(ere * ere + eim * eim), ha = sqrt(hre * hre + him * him);
        rho_imp[2 * r] = (ea / ha) * (ea / ha) / (omega * ORC_MU0);
        rho_imp[2 * r + 1] = ea / ha;   /* |e_abs / h_abs| */
    }
}

/* calcimpedance.for:163-171: quadrant rule, then the near-axis overrides in
 * the reference's order (a later match wins).  Where nothing matches
 * (both parts exactly 0) the reference keeps the previous value; 0 here. */
static double mt_phase(double re, double im, int overrides)
{
    const double pi = 3.14159265358979323846264;
    double f = 0.0;
    if (re > 0.0 && im > 0.0) f = atan(im / re);
    if (re < 0.0 && im > 0.0) f = atan(im / re) + pi;
    if (re < 0.0 && im < 0.0) f = atan(im / re) - pi;
    if (re > 0.0 && im < 0.0) f = atan(im / re);
    if (overrides) {
        if (re > 0.0 && fabs(im) < 1e-15) f = 0.0;
        if (fabs(re) < 1e-15 && im > 0.0) f = pi / 2.0;
        if (re < 0.0 && fabs(im) < 1e-15) f = pi;
        if (fabs(re) < 1e-15 && im < 0.0) f = -pi / 2.0;
    }
    return f;
}

/* Determinant of the 3x3 matrix m (row-major) by the rule of Sarrus, as
 * calcimpedance.for's `minor` (:379-386). */
static double det3(const double *m)
{
    return m[0] * m[4] * m[8] + m[3] * m[7] * m[2] + m[1] * m[5] * m[6] -
           m[2] * m[4] * m[6] - m[1] * m[3] * m[8] - m[0] * m[5] * m[7];
}

/* Inverse of a 4x4 matrix by cofactors over the first-row expansion of the
 * determinant, calcimpedance.for:346-416 (makeQ, determinan). */
static void inverse4(const double *b, double *q)
{
    double cof[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double m[9];
            int k = 0;
            for (int r = 0; r < 4; r++) {
                if (r == i) continue;
                for (int c = 0; c < 4; c++)
                    if (c != j) m[k++] = b[4 * r + c];
            }
            cof[4 * i + j] = (((i + j) & 1) ? -1.0 : 1.0) * det3(m);
        }
    double det = 0.0;
    for (int j = 0; j < 4; j++) det += b[j] * cof[j];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) q[4 * j + i] = cof[4 * i + j] / det;
}

/* calcimpedance.for:125-301.  With complex fields written re + i im, the
 * real 4x4 system B u = f states E = Z H for both polarisations:
 * rows (re, im) of polarisation X then Y, unknowns (re, im) of Z_.x, Z_.y. */
void orc_mt_response(const double *e0, const double *h0, const double *e1, const double *h1,
                     double omega, double *out)
{
    const double pi = 3.14159265358979323846264;
    const double mu0 = 4.0 * pi * 1e-7;   /* calcimpedance.for:41 */
    const double deg = 180.0 / pi;
    double B[16], Q[16];
    const double *hh[2] = {h0, h1};
    for (int p = 0; p < 2; p++) {
        const double hxr = hh[p][0], hxi = hh[p][1], hyr = hh[p][2], hyi = hh[p][3];
        double *r0 = B + 8 * p, *r1 = B + 8 * p + 4;
        r0[0] = hxr; r0[1] = -hxi; r0[2] = hyr; r0[3] = -hyi;
        r1[0] = hxi; r1[1] = hxr;  r1[2] = hyi; r1[3] = hyr;
    }
    inverse4(B, Q);
    double Z[8], W[4];
    for (int c = 0; c < 3; c++) {   /* right-hand sides: Ex, Ey, Hz */
        const double f[4] = {c < 2 ? e0[2 * c] : h0[4], c < 2 ? e0[2 * c + 1] : h0[5],
                             c < 2 ? e1[2 * c] : h1[4], c < 2 ? e1[2 * c + 1] : h1[5]};
        double u[4];
        for (int i = 0; i < 4; i++) {
            u[i] = 0.0;
            for (int j = 0; j < 4; j++) u[i] += Q[4 * i + j] * f[j];
        }
        double *dst = c < 2 ? Z + 4 * c : W;
        for (int i = 0; i < 4; i++) dst[i] = u[i];
    }
    for (int i = 0; i < 8; i++) out[i] = Z[i];
    for (int i = 0; i < 4; i++) out[8 + i] = W[i];
    for (int k = 0; k < 4; k++) {
        const double re = Z[2 * k], im = Z[2 * k + 1];
        const double m = sqrt(re * re + im * im), f = mt_phase(re, im, 1);
        out[12 + k] = m;
        out[16 + k] = -f * deg;
        out[20 + k] = m * m / (mu0 * omega);
        out[24 + k] = -2.0 * f * deg;
    }
    /* calcimpedance.for:259-276: det Z = Zxx Zyy - Zxy Zyx */
    const double dre = (Z[0] * Z[6] - Z[1] * Z[7]) - (Z[4] * Z[2] - Z[5] * Z[3]);
    const double dim = (Z[0] * Z[7] + Z[1] * Z[6]) - (Z[4] * Z[3] + Z[5] * Z[2]);
    const double zmod = sqrt(sqrt(dre * dre + dim * dim));
    const double zfi = mt_phase(dre, dim, 0) / 2.0;
    out[28] = zmod * zmod / (mu0 * omega);
    out[29] = -2.0 * zfi * deg;
    for (int k = 0; k < 2; k++) {
        const double re = W[2 * k], im = W[2 * k + 1];
        out[30 + k] = sqrt(re * re + im * im);
        out[32 + k] = -mt_phase(re, im, 1) * deg;
    }
}
