// Batched double-float survey solver (survey.cu).
#pragma once
#include "assemble.cuh"

namespace mtgpu {

// per-system state, read and written by the kernels' last blocks
struct SysState {
    double2 zs, alpha, beta;
    double r_old;          // ||b||
    double residual;       // ||s_m|| (MRS-smoothed residual)
    double residual_rel;   // residual / r_old: the reference's stop quantity
    double true_rel;       // ||b - A x|| / ||b|| of the last verification
    double mrs_w;
    double eps_k;          // the inner stop threshold on residual_rel
    double bnorm;          // ||b|| of the system (FP64)
    double rnorm;          // ||b - A x|| of the last FP64 residual evaluation
    double res_next;       // ||s_m|| after this iteration's MRS step (k_update), for the stop test
    int mrs_mode;          // 0 keep s_m, 1 s_m = r, 2 s_m += w (r - s_m): the step the next k_update applies
    int xp;                // x still lacks alpha p of the last k_update (the next k_edge or the fold adds it)
    int status;            // 1 running, else MTGPU_OK / MTGPU_DIV_BY_ZERO / MTGPU_MAXITER / MTGPU_X0_NULL
    int iter;              // the reference's iteration counter
    int checks;            // true-residual verifications
    int maxiter;
    unsigned int ticket[6];  // block-completion counters (system 0 only)
};

constexpr int kRowVariant = 16;    // + slots in flight: one thread per row, both systems
constexpr int kMatFree = 32;       // matrix-free SpMV on tensor meshes (+1: two systems per thread)
constexpr int kSpmvVariants = 11;  // 0, 1, 2, 4, 8, 18, 20, 32, 33, 34, 35

// Matrix-free SpMV of a tensor (RegularMeshBuilder) mesh: K = D^T F D with D
// the edge -> face circulations and F the face mass matrix, M the edge mass
// matrix, both regenerated from per-cell weights (survey.cu)
struct MatFree {
    bool on = false;
    int nx = 0, ny = 0, nz = 0;      // lines per axis
    long long nfx = 0, nfy = 0, nfz = 0;
    unsigned *pos = nullptr;         // [nb] rows plane by plane (x-, y-, z-edges): i | j << 10 | k << 20 | d << 30
    float2 *w = nullptr;             // [6][cells] double-float wF/3 (x, y, z), wM/9 (x, y, z)
    float4 *f = nullptr;             // face circulations [faces][SP]
    float4 *g = nullptr;             // face mass applied to them, F f [faces][SP] (variant 35)
    double check = -1.0;             // set-up check: max |A_mf s - A s| / max |A s|
    bool lattice = false;            // Dirichlet edges follow the lattice rule (always, when on)
    bool tiled = false;              // variant 34 equals variant 32 bit for bit
    bool tile_checked = false;       // ... and that was checked (on first request)
    bool gface = false;              // the D^T (F f) form agrees with variant 32 (variant 35)
    void release();
};

struct Survey {
    const ParamMatrix *P = nullptr;
    cudaStream_t st = nullptr;
    int nb = 0, S = 0, SP = 1;
    int grid_rows = 0, grid_nodes = 0;           // work bounds (blocks that have rows)
    int g_init = 0, g_node = 0, g_edge = 0, g_update = 0, g_spmv = 0, g_true = 0;  // launch grids
    int g_node_lat = 0;
    bool g_lat = false;            // G is the lattice's (k_node_lat computes its entries)
    int dir = 0;                   // sweep direction of the last launch (kernels alternate)
    // SpMV variant (autotuned): 0 x and matrix slots staged in shared memory per
    // tile, 1 x staged only, 2/4/8 gathers from global memory with that many slots in flight,
    // kRowVariant + 2/4 (two systems only) one thread per row for both systems
    int ch = 4;
    // SpMV tiles: T consecutive SELL slices, their distinct columns, per-slot local indices
    int tile_T = 1, ntiles = 0, tile_smem = 0, tile_smem_x = 0, g_spmv_t = 0, g_spmv_tx = 0;
    bool tiles_built = false;        // the stored matrix's tiles (variants 0, 1) were built
    int *uoff = nullptr, *ucol = nullptr;
    unsigned short *lc = nullptr, *lr = nullptr;
    float tune_ms[kSpmvVariants] = {};   // SpMV times of the variants 0, 1, 2, 4, 8, 18, 20, 32, 33, 34, 35
    bool autotuned = false;              // the variant was chosen by this set-up's timing
    MatFree mf;
    int g_mff = 0, g_mfe = 0;                    // matrix-free launch grids (faces, edges)
    int g_mft = 0;                               // tiled matrix-free launch grid (variant 34)
    int g_mfg = 0, g_mfe3 = 0;                   // face-mass and edge grids (variant 35)
    int mft[7] = {};                             // its tiles x, y, z chunks, groups, planes per chunk, tile columns x, y
    Folded G;                                    // pattern of G and G^T
    float2 *kc = nullptr, *mc = nullptr, *kr = nullptr;   // double-float K and M per slot
    float *gv32 = nullptr, *tv32 = nullptr;      // values of G and G^T (+-1/2, exact in FP32)
    float4 *da = nullptr, *ds = nullptr;         // 1/diag(A_k), 1/diag(G A_k G^T): [row][SP]
    float2 *omega = nullptr;                     // double-float omega_k
    double *omega64 = nullptr;
    double *gkg = nullptr, *gmg = nullptr;       // FP64 diag(G K G^T), diag(G M G^T)
    SysState *sys = nullptr, *hsys = nullptr;
    float4 *b = nullptr, *x = nullptr, *r = nullptr, *s = nullptr, *p = nullptr, *a = nullptr,
           *z = nullptr, *w = nullptr, *sm = nullptr;     // [row][SP]
    float4 *h = nullptr;                          // [node][SP]
    // the fused preconditioner of tensor meshes (prec_tile.cuh): its launch
    // grid, tiles x, y, z chunks, groups, planes per chunk, and the second
    // buffer of a (read and written in different buffers, alternating)
    bool prec_tile = false;
    int g_pt = 0, pt[5] = {};
    float prec_ms[2] = {};                        // set-up timing: ms per iteration unfused, fused
    float4 *a2 = nullptr;
    double2 *b64 = nullptr, *xacc = nullptr;      // FP64 b and accumulated x: [row][SP]
    int *all_on = nullptr;                        // 32 flags, all set
    double *partials = nullptr;
    int pblocks = 0;                              // blocks the partial-sum buffer holds
    cudaGraphExec_t graph = nullptr;
    int graph_iters = 0;
    double eps = 1e-8;
    void release();
};

// whether SpMV variant v can run on this survey: the tiled ones need their
// tiles to fit shared memory, the row-per-thread ones a two-system batch
inline bool spmv_variant_available(const Survey &V, int v)
{
    if (v == 0 || v == 1) return V.ntiles > 0;
    if (v == 2 || v == 4 || v == 8) return true;
    if (v == kRowVariant + 2 || v == kRowVariant + 4) return V.SP == 2;
    if (v == kMatFree) return V.mf.on;
    if (v == kMatFree + 1) return V.mf.on && V.SP >= 2;
    if (v == kMatFree + 2) return V.mf.on && V.mf.tiled && V.g_mft > 0 && V.g_mft <= V.pblocks;
    if (v == kMatFree + 3) return V.mf.on && V.mf.gface;
    return false;
}

// kernels an SpMV launch adds to the iteration's one: the face kernels of
// the matrix-free forms
inline int spmv_extra_launches(int v)
{
    return v == kMatFree || v == kMatFree + 1 || v == kMatFree + 3 ? 1 : 0;
}

// The host side of the matrix-free set-up (the tables themselves are
// checked and built from the device copies of the mesh)
struct MatFreeMesh {
    const double *xyz = nullptr;       // [kuzlov][3]: the node lines
    int nver_stride = 14;
    const int *nvkat = nullptr;        // [kpar]
    std::vector<double> mu, sigma;     // per material: mu3d * MU_0, sigma3d
    // the survey's M holds omega_true sigma C (a host SLAE at one frequency,
    // solved with omega = 1): omega_true is read from the SLAE's diagonal
    const int *idi = nullptr;          // block diagonal of that SLAE (lower storage)
    const double *di = nullptr;
};

// a: the assembly (host mesh copies) when the survey is built from one, or
// mfm: the mesh of a host SLAE; on a tensor mesh either enables the
// matrix-free SpMV variant
// pin_variant >= 0 (and available): that SpMV variant instead of the
// set-up autotuning
int survey_setup(const ParamMatrix &P, const mtgpu_mesh_desc &mesh, int S, const double *omega,
                 Survey &V, cudaStream_t st, const mtgpu_assembly_s *a = nullptr,
                 const MatFreeMesh *mfm = nullptr, int pin_variant = -1);
// b, x: system-major FP64 [S][nb] complex; x is the initial guess in and the
// solution out.  verify: continue until the true residual is below eps too.
int survey_solve(Survey &V, const double2 *b_sys_major, double2 *x_sys_major, double eps,
                 int maxiter, int verify, int iters_per_launch, mtgpu_survey_stats *stats);
// host state of one batch's solve (survey_begin .. survey_finish)
struct SurveyRun {
    double2 *x_out = nullptr;
    double eps = 1e-8;
    int maxiter = 0, verify = 0, ipl = 16;
    int *d_flag = nullptr;
    std::vector<int> flag = std::vector<int>(32, 0), cont = std::vector<int>(32, 0),
                     final_ = std::vector<int>(32, 0), stalled = std::vector<int>(32, 0),
                     best_it = std::vector<int>(32, 0);
    std::vector<double> last_true = std::vector<double>(32, 1e300),
                        best = std::vector<double>(32, 1e300);
    long long guard = 0, guard_max = 0;
    bool launched = false, done = false;
    void release();
};
int survey_begin(Survey &V, const double2 *b_sys_major, double2 *x_sys_major, double eps,
                 int maxiter, int verify, int iters_per_launch, SurveyRun &R);
int survey_launch(Survey &V, SurveyRun &R);
int survey_collect(Survey &V, SurveyRun &R);
// stats of the batch's systems at stats arrays [stat_offset ..]
int survey_finish(Survey &V, SurveyRun &R, mtgpu_survey_stats *stats, int stat_offset);
int survey_spmv_timed(Survey &V, int reps, float *ms);
int survey_spmv(Survey &V, const double2 *x_sys_major, double2 *y_sys_major);
int survey_iter_timed(Survey &V, int reps, float *ms);
// kernels one iteration launches
inline int iteration_launches(const Survey &V)
{
    return (V.prec_tile ? 3 : (V.G.m > 0 ? 4 : 3)) + spmv_extra_launches(V.ch);
}
int survey_set_variant(Survey &V, int variant);
// builds what `variant` needs beyond the set-up (on its first request);
// spmv_variant_available tells afterwards whether it can run
int survey_prepare_variant(Survey &V, int variant);

}  // namespace mtgpu
