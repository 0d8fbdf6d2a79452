/*
 * libmtgpu — GB300-native (sm_103a) solve stage of the MTCalc 3-D
 * magnetotelluric modeller: the COCR solver for complex-symmetric systems with
 * the folded preconditioner, on the 2x2-block SLAE format of the reference
 * (kiselev2013/MTCalc_with_DFP_COCR).
 *
 * Plain C ABI: plain pointers and sizes, no exceptions, every call returns an
 * int status.  Reference citations are paths inside the reference repository.
 *
 * Status codes.  The solver codes are the reference's RCI codes
 * (Code/COCR_FP/rci.h:23-42); library failures use values below -100.
 */
#ifndef MTGPU_H
#define MTGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define MTGPU_OK 0                 /* REQ_OK: converged                         */
#define MTGPU_X0_NULL (-1)         /* REQ_X0_NULL: the initial guess solves A x = b */
#define MTGPU_DIV_BY_ZERO (-2)     /* REQ_DIV_BY_ZERO: (a, w) = 0 breakdown     */
#define MTGPU_MAXITER (-3)         /* REQ_MAXITER: iteration limit reached      */
#define MTGPU_ERR_ARG (-101)       /* invalid argument                           */
#define MTGPU_ERR_CUDA (-102)      /* a CUDA call failed (see mtgpu_last_error) */
#define MTGPU_ERR_IO (-103)        /* a file could not be read or written        */
#define MTGPU_ERR_UNSUPPORTED (-104)
#define MTGPU_ERR_TIMEOUT (-105)   /* a bounded device wait gave up              */

/* Text of the last library error of the calling process. */
const char *mtgpu_last_error(void);

/* Number of kernels this library has launched in this process (graph
 * launches count every kernel node they contain). */
unsigned long long mtgpu_kernel_launches(void);

/* ------------------------------------------------------------------------
 * Drop-in solver: replaces PCOCR::PCOCR_2x2_Folded
 * (Code/COCR_FP/pcocr.h:27-31, Code/COCR_FP/pcocr.cpp:40-126).
 *
 * Same arguments, meaning and ownership, all host pointers, 0-based arrays:
 *   n          2 * number of edges (real length of pr and x)
 *   ig, jg, idi, ijg, di, gg   lower-triangle 2x2-block SLAE
 *   pr         right-hand side, x initial guess in / solution out
 *   eps, maxiter   stop at smoothed relative residual < eps (rci.cpp:66-75)
 *   y_omp      the reference's OpenMP scratch; unused here (may be NULL)
 *   kpar ... is_node_bound   mesh data of the folded preconditioner
 * Returns MTGPU_OK / MTGPU_X0_NULL / MTGPU_DIV_BY_ZERO / MTGPU_MAXITER as the
 * reference does, or an MTGPU_ERR_* code.  Like the reference it writes the
 * `kit` file ("r=%e\teps=%e\tkit=%d\ttime=%lf sec") in the current directory
 * (Code/COCR_FP/base_solver.cpp:181-200).
 * ---------------------------------------------------------------------- */
int mtgpu_pcocr_2x2_folded(int n, int *ig, int *jg, int *idi, int *ijg, double *di,
                           double *gg, double *pr, double *x, double eps, int maxiter,
                           double *y_omp, int kpar, int n_edges_c, int n_nodes_c,
                           double (*xyz)[3], int *nvkat, int (*nver)[14], double *sigma3d,
                           int (*edges)[2], int *ig_t, int *jg_t, double *gg_t,
                           int *is_node_bound);

typedef struct {
    int iterations;            /* the reference's `iter` at exit              */
    double residual_rel;       /* smoothed relative residual of the stop test */
    double true_residual_rel;  /* ||b - A x|| / ||b|| of the returned x (FP64) */
    double setup_seconds;      /* upload, format conversion, preconditioner   */
    double solve_seconds;      /* COCR iterations                             */
    int status;
    int spmv_variant;          /* double-float path: the SpMV variant used
                                  (see mtgpu_survey_tuning); -1 otherwise    */
    double matfree_check;      /* double-float path: the matrix-free set-up
                                  check max|A_mf s - A s| / max|A s| (the
                                  variant is offered below 1e-9); -1 when the
                                  mesh is not a tensor mesh or xyz is NULL   */
} mtgpu_solve_stats;

typedef struct {
    /* 0: stop where the reference stops (MRS-smoothed residual < eps).
     * 1: after that, keep iterating until the true residual ||b-Ax||/||b||
     *    is below eps as well (checked on the GPU in FP64). */
    int stop_on_true_residual;
    /* iterations per CUDA-graph launch between host status checks (0: 16) */
    int iterations_per_launch;
    /* 1: run the same algorithm in double-float arithmetic on the FP32 pipes
     * (the batched survey solver with one system; a system it cannot
     * finish continues in FP64, see the survey solver); 0: FP64. */
    int double_float;
} mtgpu_solve_opts;

/* Same as mtgpu_pcocr_2x2_folded with options and statistics and without
 * writing `kit`.  opts and stats may be NULL.  sigma3d: the preconditioner
 * uses only its non-zero pattern (the reference passes 0/1 flags,
 * HarmVect3d.cpp:247-316).  With double_float, when sigma3d holds the
 * materials' conductivities, xyz the node coordinates and the mesh is a
 * tensor mesh in RegularMeshBuilder's numbering, the solve may use the
 * matrix-free SpMV (mu taken as MU_0, omega read from the SLAE's diagonal):
 * it is offered only if a set-up product agrees with the SLAE's to 1e-9
 * (stats->matfree_check), otherwise the stored matrix is used. */
int mtgpu_pcocr_2x2_folded_ex(int n, const int *ig, const int *jg, const int *idi,
                              const int *ijg, const double *di, const double *gg,
                              const double *pr, double *x, double eps, int maxiter,
                              int kpar, int n_edges_c, int n_nodes_c, const double *xyz,
                              const int *nvkat, const int *nver14, const double *sigma3d,
                              const int *edges2, const int *ig_t, const int *jg_t,
                              const double *gg_t, const int *is_node_bound,
                              const mtgpu_solve_opts *opts, mtgpu_solve_stats *stats);

/* y = A x on host buffers; replaces Block_2x2_solver::Mult_MV_block_2x2
 * (Code/COCR_FP/block_2x2_solver.cpp:73-173).  x, y: 2*nb doubles. */
int mtgpu_mult_mv_block_2x2(int nb, const int *ig, const int *jg, const int *idi,
                            const int *ijg, const double *di, const double *gg,
                            const double *x, double *y);

/* y = A x on DEVICE buffers, allocating no device memory.  No counterpart in
 * the reference.  For callers that manage all GPU memory themselves (a
 * framework's caching allocator, an application that sizes every buffer up
 * front) and cannot let a library call cudaMalloc/cudaFree, which
 * synchronise the device and fail once the caller's pool holds the memory.
 * Same storage and result as mtgpu_mult_mv_block_2x2, 0-based device arrays.
 * Limit: nb <= 1048576 edges; larger nb returns MTGPU_ERR_ARG.  The work uses
 * a 16 MiB static device scratch array that every GPU loading the library
 * holds until exit and that all calls share: calls whose kernels overlap on
 * the GPU (e.g. on two streams at once) race on it.  The first call on a
 * device looks the array's address up for that device and keeps it; calls
 * after cudaDeviceReset (which may reload the module elsewhere) are not
 * supported.  The call only enqueues work on `stream` (a cudaStream_t,
 * NULL = default stream): synchronise before reading d_y or *d_status.
 * The kernels check the index arrays they cannot see from the host: if ig,
 * idi or ijg does not start at 0 (1-based arrays), nothing else is read, y is
 * left unspecified and *d_status gets MTGPU_NOALLOC_NOT_ZERO_BASED; an entry
 * whose column is not below its row, or whose block is neither 1 nor 2
 * doubles, is skipped and sets MTGPU_NOALLOC_BAD_ENTRY.  d_status is one
 * device int of the caller (0 = every entry used), or NULL. */
#define MTGPU_NOALLOC_NOT_ZERO_BASED 1
#define MTGPU_NOALLOC_BAD_ENTRY 2
int mtgpu_mult_mv_block_2x2_noalloc(int nb, const int *d_ig, const int *d_jg, const int *d_idi,
                                    const int *d_ijg, const double *d_di, const double *d_gg,
                                    const double *d_x, double *d_y, int *d_status, void *stream);

/* Folded preconditioner on host buffers: BuildGMatrix + BuildDiagComplex +
 * ApplyPreconditionerComplex (Code/COCR_FP/FoldedPreconditioner.cpp:68-259,
 * 473-574, 578-630).  y = D_A x + G^T D_S G x.  When diag_a (2*nb doubles)
 * and diag_gagt (2*m doubles, m returned in *m_out) are not NULL they receive
 * 1/diag(A) and 1/diag(G A G^T). */
int mtgpu_folded_apply(int nb, const int *ig, const int *jg, const int *idi,
                       const int *ijg, const double *di, const double *gg,
                       int kpar, int n_nodes_c, const int *nvkat, const int *nver14,
                       const double *sigma3d, const int *edges2, const int *ig_t,
                       const int *jg_t, const double *gg_t, const int *is_node_bound,
                       const double *x, double *y, int *m_out, double *diag_a,
                       double *diag_gagt);

/* ------------------------------------------------------------------------
 * Device-resident solver context: the matrix (SELL-32 full storage) and the
 * folded preconditioner live in GPU memory; right-hand sides and solutions
 * are device pointers.  This is the GB300-native form of the drop-in above
 * (the drop-in is create + solve + destroy around host copies).
 * ---------------------------------------------------------------------- */
typedef struct mtgpu_cocr_s mtgpu_cocr;

/* Build a context.  `on_device` = 1: the SLAE arrays are device pointers;
 * 0: host pointers (copied).  The mesh arrays are always host pointers.
 * stream: a cudaStream_t (NULL = legacy default stream). */
int mtgpu_cocr_create(int nb, int nnz_lower, const int *ig, const int *jg, const int *idi,
                      const int *ijg, const double *di, const double *gg, int on_device,
                      int kpar, int n_nodes_c, const int *nvkat, const int *nver14,
                      const double *sigma3d, const int *edges2, const int *ig_t,
                      const int *jg_t, const double *gg_t, const int *is_node_bound,
                      void *stream, mtgpu_cocr **out);

/* Solve A x = b with x (device, 2*nb doubles) as initial guess. */
int mtgpu_cocr_solve(mtgpu_cocr *ctx, const double *d_b, double *d_x, double eps,
                     int maxiter, const mtgpu_solve_opts *opts, mtgpu_solve_stats *stats);

/* y = A x and y = M^{-1} x on device vectors (2*nb doubles). */
int mtgpu_cocr_spmv(mtgpu_cocr *ctx, const double *d_x, double *d_y);
int mtgpu_cocr_precond(mtgpu_cocr *ctx, const double *d_x, double *d_y);

/* Time `reps` back-to-back SpMV launches y = A x on the context's stream
 * with CUDA events; *ms receives the total device time.  For measurement. */
int mtgpu_cocr_spmv_timed(mtgpu_cocr *ctx, const double *d_x, double *d_y, int reps, float *ms);

/* Sizes of the device matrix: stored complex and real entries (without
 * padding) and the number of preconditioner nodes m. */
int mtgpu_cocr_info(const mtgpu_cocr *ctx, long long *nnz_complex, long long *nnz_real,
                    int *m_nodes);

void mtgpu_cocr_destroy(mtgpu_cocr *ctx);

/* ------------------------------------------------------------------------
 * Device assembly: replaces BuildMatrix (Code/BuildMatrix/HarmVect3d.cpp:74-138:
 * T_Portrait::Gen_Portrait/Gen_idi_ijg, VecBlockSLAE::AsmBlockSLAE,
 * Bound_cond_vec_harm::SetHomogenDirichletCond).  The matrix is held on the
 * GPU in the frequency-independent form A(omega) = K + i omega M (K = sum
 * B/mu, M = sum sigma C over the cells, Dirichlet rows/columns applied), so
 * one assembly serves every frequency and polarisation of a survey.
 * ---------------------------------------------------------------------- */
typedef struct {
    int kuzlov, kpar, nb, n_materials;
    const double *xyz;        /* [kuzlov][3]                                   */
    const int *nver;          /* [kpar][nver_stride], 8 nodes used (0-based)   */
    int nver_stride;          /* 14 in nver.dat                                */
    const int *ed;            /* [kpar][ed_stride], 12 edges used (0-based)    */
    int ed_stride;            /* 25 in edges.dat                               */
    const int *edges;         /* [nb][2] node pairs (0-based)                  */
    const int *nvkat;         /* [kpar] material (0-based)                     */
    const double *mu;         /* [n_materials] mu3d * MU_0                     */
    const double *mu0;        /* may be NULL; must equal mu                    */
    const double *sigma;      /* [n_materials] sigma3d                         */
    const double *sigma0;     /* [n_materials] normal-field conductivity       */
    const double *dpr, *dpr0; /* may be NULL; must be 0 (no displacement term) */
    int n_bound;              /* boundary nodes (l13d.dat, 0-based)            */
    const int *bound_nodes;
} mtgpu_fem_mesh;

typedef struct mtgpu_assembly_s mtgpu_assembly;

int mtgpu_assembly_create(const mtgpu_fem_mesh *mesh, mtgpu_assembly **out);

/* The same assembly for a regular (tensor-product) mesh given by its node
 * lines x[nx], y[ny], z[nz] (ascending): the mesh tables (node coordinates,
 * cell nodes and edges, edge nodes, Dirichlet flags of the outer surface)
 * are generated on the device with RegularMeshBuilder's numbering
 * (Code/RegularMeshBuilder/main.cpp:923-1032: nodes x fastest, edges per
 * node +x, +y, +z; the outer surface Dirichlet, :1706-1736) instead of being
 * built and uploaded by the caller.  cell_material[(nx-1)(ny-1)(nz-1)]
 * (0-based, cells x fastest); mu, sigma, sigma0 per material as in
 * mtgpu_fem_mesh.  The result equals mtgpu_assembly_create's on the tables
 * RegularMeshBuilder writes for the same lines. */
int mtgpu_assembly_create_regular(int nx, int ny, int nz, const double *x, const double *y,
                                  const double *z, const int *cell_material, int n_materials,
                                  const double *mu, const double *sigma, const double *sigma0,
                                  mtgpu_assembly **out);

/* Sizes of the assembled system: full-storage complex/real entries, and the
 * lower-triangle block format (nnz_lower = ig[nb], gg_len = ijg[nnz_lower]). */
int mtgpu_assembly_info(const mtgpu_assembly *a, long long *nnz_complex, long long *nnz_real,
                        int *nnz_lower, long long *gg_len);

/* The SLAE of one frequency nu [Hz] and polarisation alfa (1: x, 0: y) in the
 * reference's 0-based lower-triangle block format, into host arrays sized by
 * mtgpu_assembly_info: ig[nb+1], jg[nnz_lower], idi[nb+1], ijg[nnz_lower+1],
 * di[2 nb], gg[gg_len], pr[2 nb].  z1d/usin/ucos: the 1-D normal field table
 * (Harm1D's usin.dat/ucos.dat) of that frequency. */
int mtgpu_assembly_block2x2(mtgpu_assembly *a, double nu, int alfa, int n1d, const double *z1d,
                            const double *usin, const double *ucos, int *ig, int *jg, int *idi,
                            int *ijg, double *di, double *gg, double *pr);

/* Right-hand sides of S systems into device memory d_rhs[S][2 nb]
 * (re/im interleaved).  usin/ucos: host [S][n1d] tables on the shared z1d. */
int mtgpu_assembly_rhs(mtgpu_assembly *a, int S, const double *nu, const int *alfa, int n1d,
                       const double *z1d, const double *usin, const double *ucos,
                       double *d_rhs);

/* COCR context for A(2 pi nu) built from the device assembly: no matrix
 * crosses PCIe.  stream: a cudaStream_t or NULL. */
int mtgpu_cocr_create_from_assembly(mtgpu_assembly *a, double nu, void *stream,
                                    mtgpu_cocr **out);

/* Self-check of the solver set-up: builds the folded preconditioner's G
 * and G^T for the assembly's mesh on the device (as every solver set-up
 * does) and by the host construction, and sets *equal = 1 if they agree
 * entry for entry (row pointers, columns, values, order), else 0. */
int mtgpu_assembly_check_preconditioner(mtgpu_assembly *a, int *equal);

void mtgpu_assembly_destroy(mtgpu_assembly *a);

/* ------------------------------------------------------------------------
 * Batched survey solver: up to 32 systems (frequencies x polarisations,
 * CalcStarter's loop in Code/CalcStarter/main.cpp:311-325) sharing one device
 * assembly are solved together, one lane per system, with the reference's
 * COCR + folded preconditioner + MRS stop test per system.  The arithmetic is
 * double-float (pairs of FP32 numbers, 48-bit significand) on the FP32
 * pipes, which GB300 runs at 64x its FP64 rate; the iteration follows the
 * FP64 algorithm iteration for iteration.  The solution is accumulated in
 * FP64 (group updates every 16 iterations) and true residuals are evaluated
 * in FP64 from the FP64 matrix.  A system the double-float iteration cannot
 * finish (its smoothed residual stalls: very low frequencies on fine meshes,
 * where omega sigma_air is ~1e-13 of the curl-curl scale) is finished by the
 * FP64 COCR: from its double-float solution when that is within 100 eps of
 * the target, else from x = 0.  No counterpart in the reference,
 * which solves the systems one by one in FP64.
 * ---------------------------------------------------------------------- */
typedef struct mtgpu_survey_s mtgpu_survey;

#define MTGPU_SURVEY_MAX_SYSTEMS 256

typedef struct {
    int status[MTGPU_SURVEY_MAX_SYSTEMS];          /* MTGPU_OK / MTGPU_MAXITER / ... per system */
    int iterations[MTGPU_SURVEY_MAX_SYSTEMS];      /* double-float iterations per system       */
    int verifications[MTGPU_SURVEY_MAX_SYSTEMS];   /* true-residual evaluations per system     */
    int fp64_iterations[MTGPU_SURVEY_MAX_SYSTEMS]; /* iterations of the FP64 re-solve (0: none) */
    double true_residual_rel[MTGPU_SURVEY_MAX_SYSTEMS]; /* final ||b - A x|| / ||b||           */
    double residual_rel[MTGPU_SURVEY_MAX_SYSTEMS]; /* last smoothed (stop-test) residual       */
    double seconds;                                /* host wall time of the solve              */
} mtgpu_survey_stats;

/* S systems (1 <= S <= MTGPU_SURVEY_MAX_SYSTEMS) with frequencies nu[S] [Hz]
 * on assembly a; stream: a cudaStream_t (its work is waited for before a
 * solve) or NULL.  The systems are solved in batches of up to 32 (one lane
 * per system), each batch on a stream of its own, the batches' CUDA graphs
 * launched in turn so that they run side by side. */
int mtgpu_survey_create(mtgpu_assembly *a, int S, const double *nu, void *stream,
                        mtgpu_survey **out);

/* A survey over nmesh meshes (uneven sizes): S[m] systems on assembly a[m],
 * nu[] the frequencies of all systems, mesh by mesh.  The systems' vectors
 * are packed one after the other: system k's 2 nb(k) doubles start at
 * offset_k = sum over j < k of 2 nb(j) in d_b, d_x (mtgpu_survey_info gives
 * the offsets).  Each mesh's systems form their own batches; all batches
 * run side by side as in mtgpu_survey_create.  No counterpart in the
 * reference, which runs every mesh's systems one by one. */
int mtgpu_survey_create_multi(int nmesh, mtgpu_assembly *const *a, const int *S, const double *nu,
                              void *stream, mtgpu_survey **out);

/* Number of systems, of batches, and the S + 1 packing offsets (doubles; any
 * pointer may be NULL). */
int mtgpu_survey_info(const mtgpu_survey *s, int *S, int *batches, long long *offsets);

/* d_b: device right-hand sides of all systems, packed by mtgpu_survey_info's
 * offsets ([S][2 nb] on one mesh; e.g. from mtgpu_assembly_rhs);
 * d_x: the same layout, initial guesses in, solutions out.  Each system stops
 * when its MRS-smoothed relative residual is below eps (the reference rule,
 * Code/COCR_FP/rci.cpp:66-75); with verify = 1 it then also continues until
 * ||b - A x|| / ||b|| < eps.  maxiter: per-system iteration limit (double-float
 * and FP64 re-solve iterations together). */
int mtgpu_survey_solve(mtgpu_survey *s, const double *d_b, double *d_x, double eps, int maxiter,
                       int verify, mtgpu_survey_stats *stats);

/* Time `reps` launches of the batched double-float SpMV (the first batch's
 * systems) as the
 * iteration launches it (z = A s with the MRS tail: r read, s_m read and
 * written), with CUDA events on the survey's stream; *ms receives the total.
 * It overwrites the survey's work vectors; a solve re-initialises them. */
int mtgpu_survey_spmv_timed(mtgpu_survey *s, int reps, float *ms);

/* y_k = A_k x_k = (K + i omega_k M) x_k for every system of the survey, with
 * the SpMV variant in use (double-float arithmetic; x and y FP64 device
 * [S][2 nb]).  No counterpart in the reference (Mult_MV_block_2x2,
 * Code/COCR_FP/block_2x2_solver.cpp:73-173, applies one system's stored
 * matrix).  It overwrites the survey's work vectors; a solve
 * re-initialises them. */
int mtgpu_survey_spmv(mtgpu_survey *s, const double *d_x, double *d_y);

/* The SpMV variant the set-up autotuning chose for the first batch (0: x segments and matrix
 * slots staged in shared memory per tile of slices; 1: x segments staged
 * only; 2, 4, 8: slots in flight per thread, gathers from global memory;
 * 18, 20: two-system batches only, one thread per row for both systems with
 * 2 or 4 slots in flight; 32: matrix-free, tensor meshes only: the curl-curl
 * part as D^T F D (edge -> face circulations, face mass matrix) and the mass
 * part regenerated from six weights per cell instead of the stored matrix;
 * 33: the same with two systems per thread, batches of 2 or more; 34: the
 * same operator in one kernel per launch, a block marching through the node
 * planes of its tile with the edge values and face circulations in shared
 * memory, bit-for-bit equal to 32; 35: the curl-curl part as D^T (F f), the
 * face mass matrix applied once per face and each row the signed sum over
 * its 4 faces, enabled where its set-up product agrees with 32's to 1e-12)
 * and the times it measured for the variants 0, 1, 2, 4, 8, 18, 20, 32, 33,
 * 34, 35 (ms[11]: ms
 * per whole iteration with that variant, so that each SpMV sees the cache as
 * the other kernels of an iteration leave it; 0 where a variant was not
 * available). */
int mtgpu_survey_tuning(const mtgpu_survey *s, int *variant, float *ms);
/* The environment variable MTGPU_SPMV_VARIANT, when it names a variant
 * available for the survey, replaces the autotuning at mtgpu_survey_create
 * (for profiler runs: a profiler serialises and cold-starts every launch, and
 * would make the autotuning choose differently from a plain run). */

/* Pins the SpMV variant (0, 1, 2, 4, 8, 18, 20, 32, 33, 34 or 35) instead of the
 * autotuned choice.  The stored-matrix variants sum the same products in the
 * same order; the matrix-free one computes the same operator in another
 * order (it is enabled only where a set-up product agrees with the stored
 * matrix's to 1e-9).  MTGPU_ERR_ARG if the variant is unknown or unavailable
 * for this survey (0 and 1 need their tiles to fit shared memory, 18 and 20
 * two systems, 32 a survey created from an assembly of a tensor mesh with
 * RegularMeshBuilder's numbering and all outer nodes Dirichlet, 33 that and
 * at least two systems, 34 that and no Dirichlet node inside the mesh, 35 a
 * matrix-free survey whose set-up check passed). */
int mtgpu_survey_set_spmv_variant(mtgpu_survey *s, int variant);

/* Whether the first batch runs the folded preconditioner of the iteration
 * as one fused kernel (*fused = 1; on request: the environment variable
 * MTGPU_PREC_TILE=1 at mtgpu_survey_create, on tensor meshes where a set-up
 * step of it equals the node and edge kernels' bit for bit — on GB300 it
 * measured slower than them) and the set-up's ms per iteration without and
 * with it (ms[2], 0 when not requested).  No counterpart in the reference, whose
 * ApplyPreconditionerComplex (Code/COCR_FP/FoldedPreconditioner.cpp:578-630)
 * runs G x, D_S and G^T as separate loops. */
int mtgpu_survey_preconditioner(const mtgpu_survey *s, int *fused, float *ms);

void mtgpu_survey_destroy(mtgpu_survey *s);

/* ------------------------------------------------------------------------
 * Receivers and MT responses.  Replaces the direct-evaluation output of
 * Code/OutputNu (Give_out_vec_mt::Give_out_on_hex, give_out_vec_mt.cpp:
 * 101-266, with OutputVect3d::OutputFieldAtReceivers, OutputArbitrary.cpp:
 * 202-293) and the impedance program Code/calcimpedance/calcimpedance.for:
 * 125-301.  Everything is FP64 on the device; the reference's impedance step
 * is FP32.
 * ---------------------------------------------------------------------- */
typedef struct mtgpu_receivers_s mtgpu_receivers;

/* Locates nrec receivers xyz_rec[nrec][3] (host) in the assembly's mesh: each
 * goes to the lowest-numbered brick whose closed box holds it
 * (OutputArbitrary.cpp:385-500).  Receivers outside the mesh get element -1
 * and only the 1-D normal field. */
int mtgpu_receivers_create(const mtgpu_assembly *a, int nrec, const double *xyz_rec,
                           mtgpu_receivers **out);

/* nrec, receivers without an element, and (if elem != NULL) the element of
 * every receiver (host [nrec]). */
int mtgpu_receivers_info(const mtgpu_receivers *r, int *nrec, int *n_unlocated, int *elem);

/* How mtgpu_receivers_fields obtains A and curl A at the receivers:
 *  MTGPU_OUTPUT_DIRECT (the default after create): the edge basis of the
 *    receiver's brick evaluated at the receiver, the reference's direct
 *    output (GPDocSettings.vfem_direct_output, give_out_vec_mt.cpp:109-198);
 *  MTGPU_OUTPUT_SMOOTH: the reference's default output, subdomain L2-
 *    projection smoothing (give_out_vec_mt.cpp:200-237; OutputResultant3d.cpp
 *    :76-199, 293-450; Subdomain.cpp:132-661): the brick-centre values of A
 *    (per material, air skipped) and of curl A (all materials) in the
 *    receivers' bricks grown `levels` times (the reference uses 5) by the
 *    bricks sharing a node are projected onto nodal trilinear functions, and
 *    the projection is interpolated at the receiver.  Receivers are located
 *    with boxes grown by 1e-6; a receiver with no non-air brick gets A = 0.
 *    The reference solves each projection with PARDISO; here all value types
 *    of all systems are solved together on the device by conjugate gradients
 *    to a relative residual of 1e-14.  Conforming hexahedral meshes only.
 * The assembly `a` must be the one the receivers were created on and must
 * outlive them while the output is smoothed.  The adjoint functions accept
 * the direct output only. */
#define MTGPU_OUTPUT_DIRECT 0
#define MTGPU_OUTPUT_SMOOTH 1
int mtgpu_receivers_set_output(mtgpu_receivers *r, const mtgpu_assembly *a, int mode, int levels);

/* Smoothing subdomains (at most max_sub reported): subdomain 0 smooths
 * curl A over all materials (material -1), the others A over one material
 * each; their bricks and nodes, and the conjugate-gradient iterations of the
 * last mtgpu_receivers_fields call. */
int mtgpu_receivers_smoothing_info(const mtgpu_receivers *r, int max_sub, int *nsub, int *material,
                                   int *cells, int *nodes, int *iterations);

/* Total fields of S systems at the receivers: E = -i omega A + E_1d and
 * H = curl A / MU_0 + H_1d, the 1-D part on x and y only, with A the
 * anomalous potential d_x [S][2 nb] (device, re/im interleaved, e.g. the
 * solutions of mtgpu_survey_solve).  nu[S] [Hz], alfa[S] (1: x, 0: y) and the
 * 1-D tables (z1d[n1d] ascending, usin/ucos [S][n1d], host) are those given to
 * mtgpu_assembly_rhs; the 1-D field at the receiver depth follows Harm1D's
 * e2d / b2d (Code/Harm1D/divgrad_1d.cpp:290-330).  Device outputs:
 * d_e, d_h [S][nrec][3] complex (re, im); d_rho_imp [S][nrec][2]: the
 * reference's scalar rho and |Z| of `rok` / `impedance`
 * (give_out_vec_mt.cpp:247-264). */
int mtgpu_receivers_fields(mtgpu_receivers *r, int S, const double *nu, const int *alfa, int n1d,
                           const double *z1d, const double *usin, const double *ucos,
                           const double *d_x, double *d_e, double *d_h, double *d_rho_imp);

/* One MT response record (doubles) per frequency and receiver: */
#define MTGPU_MT_Z 0         /* Zxx, Zxy, Zyx, Zyy as (re, im): 8            */
#define MTGPU_MT_W 8         /* tipper Wzx, Wzy as (re, im): 4               */
#define MTGPU_MT_ZABS 12     /* |Z..|: 4                                     */
#define MTGPU_MT_ZPHASE 16   /* -arg Z.. in degrees (files Fxx ...): 4       */
#define MTGPU_MT_RHO 20      /* |Z..|^2 / (omega mu0) (files Rxx ...): 4     */
#define MTGPU_MT_RHOPHASE 24 /* -2 arg Z.. in degrees (files Fixx ...): 4    */
#define MTGPU_MT_RHOEFF 28   /* |det Z| / (omega mu0), -arg det Z degrees: 2 */
#define MTGPU_MT_WABS 30     /* |Wz.|: 2, then -arg Wz. in degrees: 2        */
#define MTGPU_MT_RECORD 34

/* MT responses of nf frequencies nu[nf] [Hz]: sys_x[f] / sys_y[f] index the
 * X- and Y-polarisation systems (0 <= index < S) of d_e, d_h [S][nrec][3]
 * from mtgpu_receivers_fields.  d_out: device [nf][nrec][MTGPU_MT_RECORD]. */
int mtgpu_mt_response(mtgpu_receivers *r, int nf, const double *nu, const int *sys_x,
                      const int *sys_y, int S, const double *d_e, const double *d_h,
                      double *d_out);

void mtgpu_receivers_destroy(mtgpu_receivers *r);

/* ------------------------------------------------------------------------
 * Adjoint gradient of the impedance misfit
 *   J = sum_{f, r} sum_{i, j in {x, y}} |Z_ij - Zobs_ij|^2
 * with respect to the log-conductivity of every cell.  No reference
 * counterpart: the reference computes forward responses only.
 * ---------------------------------------------------------------------- */

/* The adjoint right-hand sides d_src [S][2 nb] (device, zero except on the
 * receivers' bricks) = dJ/du for the anomalous potentials u of the S systems
 * (dJ = 2 Re sum_k d_src_k^T du_k), from the fields d_e, d_h of
 * mtgpu_receivers_fields and the observed impedances d_zobs (device,
 * [nf][nrec][4] complex: Zxx, Zxy, Zyx, Zyy).  Frequencies nu[nf], systems
 * sys_x[f] / sys_y[f] as in mtgpu_mt_response; every system belongs to one
 * frequency at most.  *misfit (if not NULL) receives J. */
int mtgpu_adjoint_source(mtgpu_receivers *r, int nf, const double *nu, const int *sys_x,
                         const int *sys_y, int S, const double *d_e, const double *d_h,
                         const double *d_zobs, double *d_src, double *misfit);

/* d_grad[kpar] (device) = dJ / d ln(sigma_c) for every cell c, from the
 * forward solutions d_u and the adjoint solutions d_lambda (both [S][2 nb]
 * device; A lambda_k = src_k, A being complex symmetric) of the systems
 * nu[S], alfa[S] with the 1-D tables given to mtgpu_assembly_rhs:
 *   grad_c = sigma_c sum_k -2 Re(lambda_k^T i omega_k P C_c (u_k + a0_k))
 * with C_c the cell's mass matrix, P the non-Dirichlet rows and a0_k the 1-D
 * potential as edge values.  sigma_c is the conductivity of the cell's
 * material: with one material per cell this is the per-cell gradient. */
int mtgpu_adjoint_gradient(mtgpu_assembly *a, int S, const double *nu, const int *alfa, int n1d,
                           const double *z1d, const double *usin, const double *ucos,
                           const double *d_u, const double *d_lambda, double *d_grad);

#ifdef __cplusplus
}
#endif

/* Internal: mesh arrays of the folded preconditioner bundled together. */
typedef struct {
    int kpar, n_edges_c, n_nodes_c;
    const int *nvkat, *nver14;
    const double *sigma3d;
    const int *edges2, *ig_t, *jg_t;
    const double *gg_t;
    const int *is_node_bound;
    int nver_stride;          /* 14 for the reference arrays */
} mtgpu_mesh_desc;

#endif
