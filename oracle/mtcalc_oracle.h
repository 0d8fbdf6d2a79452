/*
 * CPU oracle for the MTCalc solve stage — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithms (kiselev2013/
 * MTCalc_with_DFP_COCR, Code/COCR_FP and Code/BuildMatrix), used by the
 * tests as the checker, by bench.py as the timed CPU baseline, and by
 * smoke() to verify one small GPU solve.  The product never links it.
 *
 * Every array is 0-based and laid out as in the reference:
 *   SLAE  ig[nb+1], jg[ig[nb]], idi[nb+1], ijg[ig[nb]+1], di[idi[nb]],
 *         gg[ijg[ig[nb]]], vectors of n = 2*nb doubles (re, im interleaved)
 *   mesh  xyz[kuzlov][3], nver[kpar][14], ed[kpar][12 used of any stride],
 *         edges[nb][2], nvkat[kpar] (0-based materials)
 *
 * Parity with the reference itself is pinned by tests/golden (fixtures made
 * by running the reference programs built from source by build_ref.sh).
 */
#ifndef MTCALC_ORACLE_H
#define MTCALC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Request codes: Code/COCR_FP/rci.h:23-42. */
#define ORC_REQ_OK 0
#define ORC_REQ_X0_NULL (-1)
#define ORC_REQ_DIV_BY_ZERO (-2)
#define ORC_REQ_MAXITER (-3)

typedef struct {
    int iterations;        /* pcocr.iter at exit */
    double residual_rel;   /* the smoothed relative residual of the stop test */
    double seconds;        /* wall time of the solve incl. preconditioner setup */
} orc_stats;

/* y = A x for the symmetric 2x2-block lower storage;
 * Code/COCR_FP/block_2x2_solver.cpp:73-173 (Mult_MV_block_2x2). */
void orc_spmv_block2x2(int nb, const int *ig, const int *jg, const int *idi,
                       const int *ijg, const double *di, const double *gg,
                       const double *x, double *y, int nthreads);

/* Folded preconditioner, Code/COCR_FP/FoldedPreconditioner.cpp. */
typedef struct {
    int n, m;
    int *iptr_g, *jptr_g;   double *gg_g;    /* G    (m x n) */
    int *iptr_gt, *jptr_gt; double *gg_gt;   /* G^T  (n x m) */
    double *diag_a;         /* 1/diag(A), complex [2n] */
    double *diag_gagt;      /* 1/diag(G A G^T), complex [2m] */
    double *help;           /* [2m] */
} orc_folded;

int orc_folded_build_g(orc_folded *p, int kpar, int n_edges_c, int n_nodes_c,
                       const int *nvkat, const int *nver14, const double *sigma3d,
                       const int *edges2, const int *ig_t, const int *jg_t,
                       const double *gg_t, const int *is_node_bound);
int orc_folded_build_diag(orc_folded *p, const int *ig, const int *jg, const int *idi,
                          const int *ijg, const double *di, const double *gg);
void orc_folded_apply(const orc_folded *p, const double *x, double *y, int nthreads);
void orc_folded_free(orc_folded *p);
/* build + one apply; returns m (test helper) */
int orc_folded_apply_once(int nb, const int *ig, const int *jg, const int *idi, const int *ijg,
                          const double *di, const double *gg, int kpar, int n_nodes_c,
                          const int *nvkat, const int *nver14, const double *sigma3d,
                          const int *edges2, const int *ig_t, const int *jg_t,
                          const double *gg_t, const int *is_node_bound, const double *x,
                          double *y, double *diag_a, double *diag_gagt);

/* The whole PCOCR_2x2_Folded solve (Code/COCR_FP/pcocr.cpp:40-126 with
 * pcocr_rci.cpp:52-181, MRS.cpp:85-153, rci.cpp:66-88).  x: initial guess in,
 * solution out.  Returns an ORC_REQ_* code. */
int orc_pcocr_2x2_folded(int n, const int *ig, const int *jg, const int *idi,
                         const int *ijg, const double *di, const double *gg,
                         const double *pr, double *x, double eps, int maxiter,
                         int kpar, int n_edges_c, int n_nodes_c,
                         const int *nvkat, const int *nver14, const double *sigma3d,
                         const int *edges2, const int *ig_t, const int *jg_t,
                         const double *gg_t, const int *is_node_bound,
                         int nthreads, int iter_limit, orc_stats *st);

/* Assembly (Code/BuildMatrix): portrait, block types, local matrices, RHS and
 * homogeneous Dirichlet conditions.
 *   materials: mu3d, mu0 (already multiplied by MU_0), sigma3d, sigma0, dpr3d,
 *   dpr0 (multiplied by DPR_0), indexed by nvkat.
 * Pass 1 (orc_portrait) returns the sizes; pass 2 fills caller arrays. */
int orc_portrait(int nb, int kpar, const int *ed12, int ed_stride,
                 int *ig /* nb+1 */, int **jg_out /* malloc'ed */);
void orc_block_types(int nb, int kpar, const int *ed12, int ed_stride,
                     const int *ig, const int *jg, int *idi, int *ijg);
int orc_assemble(int nb, int kpar, const double *xyz, const int *nver14,
                 const int *ed12, int ed_stride, const int *edges2,
                 const int *nvkat, const double *mu3d, const double *mu0,
                 const double *sigma3d, const double *sigma0,
                 const double *dpr3d, const double *dpr0,
                 double nu, int alfa, int n1d, const double *z1d,
                 const double *usin, const double *ucos,
                 int kuzlov, int kt1, const int *l13d,
                 const int *ig, const int *jg, const int *idi, const int *ijg,
                 double *di, double *gg, double *pr);

/* Local brick matrices, 12x12 row-major, before the material scaling:
 * b = curl-curl (Code/BuildMatrix/T_Brick.cpp:123-290),
 * c = mass     (T_Brick.cpp:292-455). */
void orc_brick_bc(double hx, double hy, double hz, double *b, double *c);

/* Linear interpolation of a 1-D table; Code/BuildMatrix/For_Solvers.cpp:236-270. */
double orc_spline(double x, int n, const double *z, const double *v);

/* ---- receivers and MT responses ------------------------------------------ */

/* Receiver location, Code/OutputNu/OutputArbitrary.cpp:385-500
 * (FindElemForReceivers): receiver r goes to the lowest-numbered brick whose
 * closed box [xyz(nver[e][0]), xyz(nver[e][7])] holds it; -1 if none.
 * Returns the number of receivers left without an element. */
int orc_locate_receivers(int kpar, const int *nver14, const double *xyz, int nrec,
                         const double *rec, int *elem);

/* A and curl A of the edge solution v3 ([nb][2] re/im) at the receivers,
 * Code/OutputNu/T_Brick.cpp:980-1137 (basis, VectorFieldOnPar) and :1842-1918
 * with :1484-1618 (RotX/Y/ZOnPar).  a, curl: [nrec][3][2]; zero where elem < 0. */
void orc_receiver_eval(const int *nver14, const int *ed25, const double *xyz, int nrec,
                       const double *rec, const int *elem, const double *v3,
                       double *a, double *curl);

/* Derivative of a 1-D table, Code/Harm1D/divgrad_1d.cpp:90-135 (dSpline). */
double orc_dspline(double x, int n, const double *z, const double *v);

/* 1-D normal field at depth z as Harm1D writes it into e2d / b2d
 * (divgrad_1d.cpp:290-330): e, b = (x_re, y_re, z_re, x_im, y_im, z_im). */
void orc_normal_field(double z, int n1d, const double *z1d, const double *usin,
                      const double *ucos, int alfa, double omega, double *e, double *b);

/* Total receiver fields of Give_out_on_hex (Code/OutputNu/give_out_vec_mt.cpp:
 * 135-195 and 232-266), direct evaluation, MT task: E = -i omega A + E_1d,
 * H = curl A / MU_0 + B_1d / MU_0 (normal part on x, y only), and the two
 * scalars written to `rok` and `impedance`.
 * e, h: [nrec][3][2]; rho_imp: [nrec][2] (rho, |Z|); e1d, b1d: [nrec][6]. */
void orc_receiver_fields(int nrec, const double *a, const double *curl, double omega,
                         const double *e1d, const double *b1d, double *e, double *h,
                         double *rho_imp);

/* MT responses of one receiver and frequency from the X- and Y-polarisation
 * fields, Code/calcimpedance/calcimpedance.for:125-301 (in FP64; the
 * reference computes in FP32).  e0, h0, e1, h1: [3][2] complex (polarisation
 * X, Y).  out: ORC_MT_RECORD doubles, layout as mtgpu.h's MTGPU_MT_*. */
#define ORC_MT_RECORD 34
void orc_mt_response(const double *e0, const double *h0, const double *e1, const double *h1,
                     double omega, double *out);

#ifdef __cplusplus
}
#endif
#endif
