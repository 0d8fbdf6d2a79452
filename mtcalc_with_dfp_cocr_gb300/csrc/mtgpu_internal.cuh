// Internal declarations shared by the libmtgpu translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <vector>

#include "../../include/mtgpu.h"

namespace mtgpu {

// --------------------------------------------------------------- errors
#define MTGPU_TRY(expr)                                                        \
    do {                                                                       \
        cudaError_t e_ = (expr);                                               \
        if (e_ != cudaSuccess) {                                               \
            ::mtgpu::set_last_error(e_, #expr, __FILE__, __LINE__);           \
            return MTGPU_ERR_CUDA;                                             \
        }                                                                      \
    } while (0)

#define MTGPU_CHECK_ARG(cond, msg)                                             \
    do {                                                                       \
        if (!(cond)) {                                                         \
            ::mtgpu::set_last_message(msg);                                    \
            return MTGPU_ERR_ARG;                                              \
        }                                                                      \
    } while (0)

void set_last_error(cudaError_t e, const char *what, const char *file, int line);
void set_last_message(const char *msg);

constexpr int kSlice = 32;          // SELL slice height = one warp of rows
constexpr int kThreads = 256;       // default block size for row/edge kernels

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// ------------------------------------------------ device matrix (SELL-32)
// Full (both triangles) complex-symmetric matrix in sliced ELL with slice
// height 32.  Every row is split into complex slots (diagonal and parallel
// edge pairs: 16-byte values) and real slots (perpendicular pairs: 8-byte
// values).  Slot k of row (32*s + l) lives at sptr[s] + 32*k + l, so a warp
// reading one slot of its 32 rows touches one contiguous segment.
struct SellMatrix {
    int nb = 0;                 // rows (edges)
    int nslices = 0;
    long long nnz_c = 0, nnz_r = 0;          // stored entries without padding
    long long len_c = 0, len_r = 0;          // stored slots with padding
    int *d_wc = nullptr, *d_wr = nullptr;    // slice widths [nslices]
    long long *d_pc = nullptr, *d_pr = nullptr;  // slice offsets [nslices+1]
    int *d_col_c = nullptr, *d_col_r = nullptr;
    double2 *d_val_c = nullptr;
    double *d_val_r = nullptr;
    int *d_diag_slot = nullptr;   // complex slot index of the diagonal, per row
    int *d_nc = nullptr, *d_nr = nullptr;   // complex / real entries per row
    void release();
};

// Builds the SELL matrix from the reference lower 2x2-block storage that is
// already resident on the device (0-based arrays).
int sell_from_block2x2_device(int nb, const int *d_ig, const int *d_jg, const int *d_idi,
                              const int *d_ijg, const double *d_di, const double *d_gg,
                              int nnz_lower, SellMatrix &A, cudaStream_t st);

// y = A x  (x, y complex interleaved, device)
void sell_spmv(const SellMatrix &A, const double2 *x, double2 *y, cudaStream_t st);
// y = b - A x
void sell_residual(const SellMatrix &A, const double2 *b, const double2 *x, double2 *y,
                   cudaStream_t st);

// ------------------------------------------------ folded preconditioner
struct Folded {
    int n = 0, m = 0;                  // edges, interior conductive nodes
    int *d_gp = nullptr, *d_gj = nullptr;   double *d_gv = nullptr;   // G   (CSR, m rows)
    int *d_tp = nullptr, *d_tj = nullptr;   double *d_tv = nullptr;   // G^T (CSR, n rows)
    // G^T of a conforming mesh in compact form: per edge the G rows of its
    // first (-1/2) and second (+1/2) node, -1 where the node has no row;
    // null on meshes with T-matrix nodes
    int2 *d_tn = nullptr;
    double2 *d_da = nullptr;           // 1/diag(A)
    double2 *d_ds = nullptr;           // 1/diag(G A G^T)
    double2 *d_h = nullptr;            // node work vector
    void release();
};

// Host construction of G and G^T (FoldedPreconditioner.cpp:68-259 semantics),
// uploaded to the device.
int folded_build_g(const mtgpu_mesh_desc &mesh, Folded &P, cudaStream_t st);

// Device copies of the mesh tables that the set-up stages read (0-based)
struct DevMesh {
    int kpar = 0, nb = 0, nn = 0, nver_stride = 8, nmat = 0;
    const double *xyz = nullptr;            // [nn][3]; null where not needed
    const int *nver = nullptr;              // [kpar][nver_stride]
    const int *nvkat = nullptr;             // [kpar]
    const int *edges = nullptr;             // [nb][2]
    const double *sigflag = nullptr;        // [nmat]: > 0 for conductive materials
    const unsigned char *bnode = nullptr;   // [nn]: Dirichlet nodes
};
// A DevMesh over uploads of a host mesh description (or over tables
// already on the device plus the uploaded material flags); the uploads are
// freed with the object
struct DevMeshUpload {
    DevMesh view;
    int *nver = nullptr, *nvkat = nullptr, *edges = nullptr;
    double *xyz = nullptr, *sigflag = nullptr;
    unsigned char *bnode = nullptr;
    int upload(const mtgpu_mesh_desc &m, const double *xyz_host, cudaStream_t st);
    int over_device(int kpar, int nb, int nn, int nver_stride, const double *d_xyz,
                    const int *d_nver, const int *d_nvkat, const int *d_edges,
                    const unsigned char *d_bnode, const double *sigflag_host, int nmat,
                    cudaStream_t st);
    void release();
    ~DevMeshUpload() { release(); }
};
// G and G^T built on the device (same rows, entries and order as
// folded_build_g); *conforming = false, and nothing built, when an edge
// has a node beyond nn (T-matrix meshes: folded_build_g handles them)
int folded_build_g_device(const DevMesh &dm, Folded &P, cudaStream_t st, bool *conforming);
// G and G^T for a solver set-up: on the device from dm (or from an upload of
// the host mesh description when dm is null) where the mesh is conforming,
// else by the host construction
int folded_build_g_auto(const mtgpu_mesh_desc &mesh, const DevMesh *dm, Folded &P, cudaStream_t st);
// exclusive prefix sum: out[0..n] (out[n] = total), *total on the host
int dev_exclusive_scan(const int *d_in, long long n, int *d_out, long long *total, cudaStream_t st);
// D_A and D_S from the device matrix.
int folded_build_diag(const SellMatrix &A, Folded &P, cudaStream_t st);
// y = D_A x + G^T D_S G x
void folded_apply(const Folded &P, const double2 *x, double2 *y, cudaStream_t st);

// ------------------------------------------------ COCR solver state
struct Ctl;   // device control block (cocr.cu)
struct CocrSolver {
    SellMatrix A;
    Folded P;
    cudaStream_t st = nullptr;
    int nb = 0;
    int grid = 0;                 // blocks of the reduction kernels
    double2 *r = nullptr, *p = nullptr, *s = nullptr, *z = nullptr, *a = nullptr,
            *w = nullptr, *sm = nullptr;
    double *partials = nullptr;
    Ctl *ctl = nullptr;           // device
    Ctl *hctl = nullptr;          // pinned host mirror
    cudaGraphExec_t graph = nullptr;
    const void *graph_x = nullptr;
    int graph_iters = 0;
    void release();
};
int cocr_alloc(CocrSolver &S);
int cocr_solve(CocrSolver &S, const double2 *b, double2 *x, double eps, int maxiter,
               int stop_true, int iters_per_launch, mtgpu_solve_stats *stats);
void note_launches(unsigned long long k);

// ------------------------------------------------ small device helpers
__host__ __device__ inline double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// a / b with scaling against overflow (Smith's algorithm)
__host__ __device__ inline double2 cdiv(double2 a, double2 b)
{
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, d = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    const double r = b.x / b.y, d = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}

// device allocation helpers (record the failing call)
template <class T>
int dev_alloc(T **p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    MTGPU_TRY(cudaMalloc((void **)p, count * sizeof(T)));
    return MTGPU_OK;
}
template <class T>
void dev_free(T *&p)
{
    if (p) cudaFree((void *)p);
    p = nullptr;
}

}  // namespace mtgpu

// opaque handle of the C ABI
struct mtgpu_cocr_s {
    mtgpu::CocrSolver S;
    bool own_stream = false;
};

namespace mtgpu {
int make_stream(mtgpu_cocr_s *c, void *stream);
double now_seconds();

// MTGPU_TRACE=1 (environment): the phases of a set-up on stderr, each
// after a synchronisation of its stream so that device work is charged to
// the phase that launched it; MTGPU_TRACE=2: host time only, no
// synchronisation (where the host itself waits)
struct PhaseTrace {
    bool on = false, sync = true;
    cudaStream_t st;
    const char *what;
    double t0 = 0.0, last = 0.0;
    PhaseTrace(cudaStream_t s, const char *w) : st(s), what(w)
    {
        const char *e = getenv("MTGPU_TRACE");
        on = e && (*e == '1' || *e == '2');
        sync = !(e && *e == '2');
        t0 = last = now_seconds();
    }
    void mark(const char *phase)
    {
        if (!on) return;
        if (sync) cudaStreamSynchronize(st);
        const double now = now_seconds();
        fprintf(stderr, "[mtgpu] %s %-22s %8.2f ms (total %8.2f)\n", what, phase, 1e3 * (now - last),
                1e3 * (now - t0));
        last = now;
    }
};
}  // namespace mtgpu
