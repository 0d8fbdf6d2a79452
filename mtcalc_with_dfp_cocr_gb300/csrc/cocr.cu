// Preconditioned COCR for complex-symmetric systems, FP64, on the device.
//
// The recurrences are the reference's PCOCR_RCI::Run
// (Code/COCR_FP/pcocr_rci.cpp:52-181): unconjugated bilinear dots
// (base_solver.cpp:382-399), alpha = (z,s)/(a,w), beta = (z,s)_new/(z,s)_old,
// the stop test on the MRS-smoothed residual relative to ||b||
// (MRS.cpp:85-153, rci.cpp:66-75), REQ_DIV_BY_ZERO when (a,w) vanishes.
//
// One iteration is four kernels, captured into a CUDA graph several
// iterations at a time; every decision (alpha, beta, the MRS weight, the
// stop test, the iteration limit) is taken on the device by the last block
// of the kernel that finishes the reduction, so the host only looks at the
// status word between graph launches.
//   k_it_node   h = D_S G (z + beta a)                      [node gather]
//   k_it_edge   p = s + beta p, a = z + beta a,
//               w = D_A a + G^T h, (a,w)  -> alpha            [edge gather]
//   k_it_update x += alpha p, r -= alpha a, s -= alpha w,
//               MRS weight from (s_m, r - s_m), |r - s_m|^2
//   k_it_spmv   z = A s, MRS smoothing of s_m, |s_m|, (z,s)
//               -> stop test, beta
// Reductions are two-level (fixed per-block partials, then the last block
// sums them in block order), so results do not change run to run.
#include "mtgpu_internal.cuh"

namespace mtgpu {

enum : int { kRunning = 1 };

struct Ctl {
    int status;          // kRunning or a final MTGPU_* code
    int iter;            // number of the iteration in progress / at exit
    int maxiter;
    int mrs_mode;        // 0 keep s_m, 1 s_m = r, 2 s_m += w (r - s_m)
    double mrs_w;
    double eps;
    double r_old;        // ||b||
    double residual;     // ||s_m||
    double residual_rel;
    double2 alpha, beta, zs;
    double sums[4];      // scratch results of one-off reductions
    unsigned int ticket[4];
};

namespace {

constexpr int kRedThreads = 256;

// ---------------------------------------------------------- reductions
template <int N>
__device__ inline void block_sum(double (&v)[N], double *smem /* N * 32 */)
{
#pragma unroll
    for (int k = 0; k < N; k++)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; k++) smem[k * 32 + warp] = v[k];
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < N; k++) {
            v[k] = lane < nw ? smem[k * 32 + lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        }
    }
}

// Publish this block's partial sums; returns true in the one block that
// arrives last, which then holds the grid totals in v (thread 0).
template <int N>
__device__ bool grid_sum(double (&v)[N], double *partials, unsigned int *ticket)
{
    __shared__ double smem[N * 32];
    __shared__ bool last;
    block_sum<N>(v, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < N; k++) partials[(size_t)k * gridDim.x + blockIdx.x] = v[k];
        __threadfence();
        const unsigned int t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
        acc[k] = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            acc[k] += __ldcg(&partials[(size_t)k * gridDim.x + b]);
    }
    block_sum<N>(acc, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < N; k++) v[k] = acc[k];
        *ticket = 0u;
    }
    return true;
}

__device__ inline bool running(const Ctl *c) { return *(volatile const int *)&c->status == kRunning; }

// ------------------------------------------------------------ set-up
// r = b - A x is computed by the SpMV kernel; this one finishes stage 2:
// ||b||, ||r||, the x0 test (rci.cpp:79-88) and MRS initialisation s_m = r.
__global__ void __launch_bounds__(kRedThreads)
k_init_norms(int nb, const double2 *__restrict__ b, const double2 *__restrict__ r,
             double2 *__restrict__ sm, Ctl *ctl, double *partials)
{
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const double2 bv = b[i], rv = r[i];
        v[0] += bv.x * bv.x + bv.y * bv.y;
        v[1] += rv.x * rv.x + rv.y * rv.y;
        sm[i] = rv;
    }
    if (grid_sum<2>(v, partials, &ctl->ticket[0]) && threadIdx.x == 0) {
        ctl->r_old = v[0] > 0.0 ? sqrt(v[0]) : 0.0;
        ctl->residual = v[1] > 0.0 ? sqrt(v[1]) : 0.0;
        ctl->residual_rel = ctl->r_old > 0.0 ? ctl->residual / ctl->r_old : 0.0;
        ctl->beta = make_double2(0.0, 0.0);
        ctl->iter = 1;
        if (ctl->residual < 1e-30) {
            ctl->status = MTGPU_X0_NULL;
            ctl->iter = 0;
            ctl->residual_rel = 1.0;   // the RCI's initial residualRel (rci.cpp:40)
        } else if (ctl->maxiter < 1) ctl->status = MTGPU_MAXITER;
        else ctl->status = kRunning;
    }
}

// zs = (z, s) for the first iteration (stage 4 -> 5)
__global__ void __launch_bounds__(kRedThreads)
k_init_zs(int nb, const double2 *__restrict__ z, const double2 *__restrict__ s, Ctl *ctl,
          double *partials)
{
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const double2 a = z[i], c = s[i];
        v[0] += a.x * c.x - a.y * c.y;
        v[1] += a.x * c.y + a.y * c.x;
    }
    if (grid_sum<2>(v, partials, &ctl->ticket[0]) && threadIdx.x == 0)
        ctl->zs = make_double2(v[0], v[1]);
}

// ||b - A x||^2 and ||b||^2 of a residual vector already formed
__global__ void __launch_bounds__(kRedThreads)
k_norm2(int nb, const double2 *__restrict__ r, const double2 *__restrict__ b, Ctl *ctl,
        double *partials)
{
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const double2 rv = r[i], bv = b[i];
        v[0] += rv.x * rv.x + rv.y * rv.y;
        v[1] += bv.x * bv.x + bv.y * bv.y;
    }
    if (grid_sum<2>(v, partials, &ctl->ticket[0]) && threadIdx.x == 0) {
        ctl->sums[0] = v[0];
        ctl->sums[1] = v[1];
    }
}

// ------------------------------------------------------- the iteration
__global__ void __launch_bounds__(kThreads)
k_it_node(int m, const int *__restrict__ gp, const int *__restrict__ gj,
          const double *__restrict__ gv, const double2 *__restrict__ ds,
          const double2 *__restrict__ z, const double2 *__restrict__ a,
          double2 *__restrict__ h, const Ctl *ctl)
{
    if (!running(ctl)) return;
    const double2 beta = ctl->beta;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < m; v += gridDim.x * blockDim.x) {
        double hr = 0.0, hi = 0.0;
        for (int j = gp[v]; j < gp[v + 1]; j++) {
            const int e = gj[j];
            const double2 an = cadd(z[e], cmul(beta, a[e]));
            hr += gv[j] * an.x;
            hi += gv[j] * an.y;
        }
        h[v] = cmul(make_double2(hr, hi), ds[v]);
    }
}

__global__ void __launch_bounds__(kRedThreads)
k_it_edge(int n, const int *__restrict__ tp, const int *__restrict__ tj,
          const double *__restrict__ tv, const double2 *__restrict__ da,
          const double2 *__restrict__ h, const double2 *__restrict__ s,
          const double2 *__restrict__ z, double2 *__restrict__ p, double2 *__restrict__ a,
          double2 *__restrict__ w, Ctl *ctl, double *partials)
{
    if (!running(ctl)) return;
    const double2 beta = ctl->beta;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double2 pn = cadd(s[i], cmul(beta, p[i]));
        const double2 an = cadd(z[i], cmul(beta, a[i]));
        double2 wn = cmul(an, da[i]);
        for (int j = tp[i]; j < tp[i + 1]; j++) {
            const double2 hv = h[tj[j]];
            wn.x += tv[j] * hv.x;
            wn.y += tv[j] * hv.y;
        }
        p[i] = pn;
        a[i] = an;
        w[i] = wn;
        v[0] += an.x * wn.x - an.y * wn.y;
        v[1] += an.x * wn.y + an.y * wn.x;
    }
    if (grid_sum<2>(v, partials, &ctl->ticket[1]) && threadIdx.x == 0) {
        const double2 aw = make_double2(v[0], v[1]);
        if (fabs(aw.x) < 1e-40 && fabs(aw.y) < 1e-40) {
            ctl->status = MTGPU_DIV_BY_ZERO;
        } else {
            ctl->alpha = cdiv(ctl->zs, aw);
        }
    }
}

__global__ void __launch_bounds__(kRedThreads)
k_it_update(int n, const double2 *__restrict__ p, const double2 *__restrict__ a,
            const double2 *__restrict__ w, const double2 *__restrict__ sm,
            double2 *__restrict__ x, double2 *__restrict__ r, double2 *__restrict__ s, Ctl *ctl,
            double *partials)
{
    if (!running(ctl)) return;
    const double2 al = ctl->alpha;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] = cadd(x[i], cmul(al, p[i]));
        const double2 rn = csub(r[i], cmul(al, a[i]));
        r[i] = rn;
        s[i] = csub(s[i], cmul(al, w[i]));
        const double2 sv = sm[i];
        const double ux = rn.x - sv.x, uy = rn.y - sv.y;
        v[0] += sv.x * ux + sv.y * uy;
        v[1] += ux * ux + uy * uy;
    }
    if (grid_sum<2>(v, partials, &ctl->ticket[2]) && threadIdx.x == 0) {
        const double su = v[0], uu = v[1];
        const double wm = fabs(uu) < 1e-100 ? 0.0 : -su / uu;
        if (wm < 0.0) {
            ctl->mrs_mode = 0;
        } else if (wm > 1.0) {
            ctl->mrs_mode = 1;
        } else {
            ctl->mrs_mode = 2;
            ctl->mrs_w = wm;
        }
    }
}

__global__ void __launch_bounds__(kRedThreads)
k_it_spmv(int nb, const int *__restrict__ wc, const int *__restrict__ wr,
          const long long *__restrict__ pc, const long long *__restrict__ pr,
          const int *__restrict__ col_c, const double2 *__restrict__ val_c,
          const int *__restrict__ col_r, const double *__restrict__ val_r,
          const double2 *__restrict__ s, const double2 *__restrict__ r,
          double2 *__restrict__ z, double2 *__restrict__ sm, Ctl *ctl, double *partials)
{
    if (!running(ctl)) return;
    const int mode = ctl->mrs_mode;
    const double wm = ctl->mrs_w;
    double v[3] = {0.0, 0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        const int sl = i / kSlice, l = i % kSlice;
        double ar = 0.0, ai = 0.0;
        {
            const long long base = pc[sl] + l;
            const int wdt = wc[sl];
#pragma unroll 4
            for (int k = 0; k < wdt; k++) {
                const double2 vv = val_c[base + (long long)k * kSlice];
                const double2 xv = s[col_c[base + (long long)k * kSlice]];
                ar += vv.x * xv.x - vv.y * xv.y;
                ai += vv.x * xv.y + vv.y * xv.x;
            }
        }
        {
            const long long base = pr[sl] + l;
            const int wdt = wr[sl];
#pragma unroll 8
            for (int k = 0; k < wdt; k++) {
                const double vv = val_r[base + (long long)k * kSlice];
                const double2 xv = s[col_r[base + (long long)k * kSlice]];
                ar += vv * xv.x;
                ai += vv * xv.y;
            }
        }
        z[i] = make_double2(ar, ai);
        const double2 si = s[i];
        v[0] += ar * si.x - ai * si.y;
        v[1] += ar * si.y + ai * si.x;
        if (mode != 0) {
            double2 smv = r[i];
            if (mode == 2) {
                const double2 old = sm[i];
                smv = make_double2(old.x + wm * (smv.x - old.x), old.y + wm * (smv.y - old.y));
            }
            sm[i] = smv;
            v[2] += smv.x * smv.x + smv.y * smv.y;
        }
    }
    if (grid_sum<3>(v, partials, &ctl->ticket[3]) && threadIdx.x == 0) {
        if (mode != 0) ctl->residual = sqrt(v[2]);
        ctl->residual_rel = ctl->residual / ctl->r_old;
        const double2 zs_new = make_double2(v[0], v[1]);
        ctl->beta = cdiv(zs_new, ctl->zs);
        ctl->zs = zs_new;
        if (ctl->residual_rel < ctl->eps) {
            ctl->status = MTGPU_OK;
        } else {
            ctl->iter += 1;
            if (ctl->iter > ctl->maxiter) ctl->status = MTGPU_MAXITER;
        }
    }
}

}  // namespace

// ---------------------------------------------------------------- solver
void CocrSolver::release()
{
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    A.release();
    P.release();
    dev_free(r); dev_free(p); dev_free(s); dev_free(z); dev_free(a); dev_free(w); dev_free(sm);
    dev_free(partials);
    dev_free(ctl);
    if (hctl) cudaFreeHost(hctl);
    hctl = nullptr;
}

int cocr_alloc(CocrSolver &S)
{
    const int nb = S.nb;
    int dev = 0, nsm = 0;
    MTGPU_TRY(cudaGetDevice(&dev));
    MTGPU_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    // as many blocks as are resident at once (the loops are grid-stride), so
    // no block waits for a second wave
    int occ = 64;
    const void *fs[] = {(const void *)k_it_edge, (const void *)k_it_update, (const void *)k_it_spmv,
                        (const void *)k_init_norms};
    for (const void *f : fs) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, kRedThreads, 0) == cudaSuccess && b > 0)
            occ = std::min(occ, b);
    }
    S.grid = std::max(1, std::min(ceil_div(nb, kRedThreads), occ * nsm));
    int rc;
    if ((rc = dev_alloc(&S.r, nb)) || (rc = dev_alloc(&S.p, nb)) || (rc = dev_alloc(&S.s, nb)) ||
        (rc = dev_alloc(&S.z, nb)) || (rc = dev_alloc(&S.a, nb)) || (rc = dev_alloc(&S.w, nb)) ||
        (rc = dev_alloc(&S.sm, nb)) || (rc = dev_alloc(&S.partials, (size_t)4 * S.grid)) ||
        (rc = dev_alloc(&S.ctl, 1)))
        return rc;
    MTGPU_TRY(cudaMallocHost((void **)&S.hctl, sizeof(Ctl)));
    MTGPU_TRY(cudaMemsetAsync(S.ctl, 0, sizeof(Ctl), S.st));
    return MTGPU_OK;
}

static void launch_iteration(CocrSolver &S, double2 *x)
{
    const Folded &P = S.P;
    const SellMatrix &A = S.A;
    const int nb = S.nb, g = S.grid;
    if (P.m > 0)
        k_it_node<<<std::max(1, std::min(ceil_div(P.m, kThreads), g)), kThreads, 0, S.st>>>(
            P.m, P.d_gp, P.d_gj, P.d_gv, P.d_ds, S.z, S.a, P.d_h, S.ctl);
    k_it_edge<<<g, kRedThreads, 0, S.st>>>(nb, P.d_tp, P.d_tj, P.d_tv, P.d_da, P.d_h, S.s, S.z,
                                           S.p, S.a, S.w, S.ctl, S.partials);
    k_it_update<<<g, kRedThreads, 0, S.st>>>(nb, S.p, S.a, S.w, S.sm, x, S.r, S.s, S.ctl,
                                             S.partials);
    k_it_spmv<<<g, kRedThreads, 0, S.st>>>(nb, A.d_wc, A.d_wr, A.d_pc, A.d_pr, A.d_col_c,
                                           A.d_val_c, A.d_col_r, A.d_val_r, S.s, S.r, S.z, S.sm,
                                           S.ctl, S.partials);
}

static int kernels_per_iteration(const CocrSolver &S) { return S.P.m > 0 ? 4 : 3; }

static int build_graph(CocrSolver &S, double2 *x, int iters)
{
    if (S.graph) cudaGraphExecDestroy(S.graph);
    S.graph = nullptr;
    cudaGraph_t g;
    MTGPU_TRY(cudaStreamBeginCapture(S.st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < iters; k++) launch_iteration(S, x);
    MTGPU_TRY(cudaStreamEndCapture(S.st, &g));
    cudaError_t e = cudaGraphInstantiate(&S.graph, g, 0);
    cudaGraphDestroy(g);
    MTGPU_TRY(e);
    S.graph_x = x;
    S.graph_iters = iters;
    return MTGPU_OK;
}

static int sync_ctl(CocrSolver &S)
{
    MTGPU_TRY(cudaMemcpyAsync(S.hctl, S.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, S.st));
    MTGPU_TRY(cudaStreamSynchronize(S.st));
    return MTGPU_OK;
}

// true relative residual ||b - A x|| / ||b|| (FP64), via S.w as scratch
static int true_residual(CocrSolver &S, const double2 *b, const double2 *x, double *out)
{
    sell_residual(S.A, b, x, S.w, S.st);
    k_norm2<<<S.grid, kRedThreads, 0, S.st>>>(S.nb, S.w, b, S.ctl, S.partials);
    note_launches(2);
    MTGPU_TRY(cudaGetLastError());
    int rc = sync_ctl(S);
    if (rc) return rc;
    const double rr = S.hctl->sums[0], bb = S.hctl->sums[1];
    *out = bb > 0.0 ? sqrt(rr) / sqrt(bb) : 0.0;
    return MTGPU_OK;
}

int cocr_solve(CocrSolver &S, const double2 *b, double2 *x, double eps, int maxiter,
               int stop_true, int iters_per_launch, mtgpu_solve_stats *stats)
{
    const int nb = S.nb;
    if (iters_per_launch <= 0) iters_per_launch = 16;
    Ctl init{};
    init.status = kRunning;
    init.maxiter = maxiter;
    init.eps = eps;
    MTGPU_TRY(cudaMemcpyAsync(S.ctl, &init, sizeof(Ctl), cudaMemcpyHostToDevice, S.st));
    // stages 1-4 of PCOCR_RCI::Run
    sell_residual(S.A, b, x, S.r, S.st);                                    // r = b - A x
    k_init_norms<<<S.grid, kRedThreads, 0, S.st>>>(nb, b, S.r, S.sm, S.ctl, S.partials);
    folded_apply(S.P, S.r, S.s, S.st);                                      // s = M^-1 r
    MTGPU_TRY(cudaMemsetAsync(S.p, 0, sizeof(double2) * nb, S.st));
    MTGPU_TRY(cudaMemsetAsync(S.a, 0, sizeof(double2) * nb, S.st));
    MTGPU_TRY(cudaMemsetAsync(S.w, 0, sizeof(double2) * nb, S.st));
    sell_spmv(S.A, S.s, S.z, S.st);                                         // z = A s
    k_init_zs<<<S.grid, kRedThreads, 0, S.st>>>(nb, S.z, S.s, S.ctl, S.partials);
    note_launches(S.P.m > 0 ? 6 : 5);
    MTGPU_TRY(cudaGetLastError());
    int rc = sync_ctl(S);
    if (rc) return rc;

    if (S.graph == nullptr || S.graph_x != (const void *)x || S.graph_iters != iters_per_launch)
        if ((rc = build_graph(S, x, iters_per_launch))) return rc;

    const unsigned long long kpi = (unsigned long long)kernels_per_iteration(S);
    double true_rr = -1.0;
    // every launch advances at least one iteration until the status is final
    for (long long guard = 0; guard <= (long long)maxiter + 2; guard += iters_per_launch) {
        if (S.hctl->status != kRunning) {
            if (S.hctl->status == MTGPU_OK && stop_true) {
                if ((rc = true_residual(S, b, x, &true_rr))) return rc;
                if (true_rr >= eps) {
                    // keep iterating: the recurrences already hold the next
                    // iteration's z, s and beta
                    Ctl c = *S.hctl;
                    c.status = kRunning;
                    c.iter += 1;
                    if (c.iter > c.maxiter) c.status = MTGPU_MAXITER;
                    MTGPU_TRY(cudaMemcpyAsync(S.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, S.st));
                    if ((rc = sync_ctl(S))) return rc;
                    true_rr = -1.0;
                    continue;
                }
            }
            break;
        }
        MTGPU_TRY(cudaGraphLaunch(S.graph, S.st));
        note_launches(kpi * (unsigned long long)iters_per_launch);
        if ((rc = sync_ctl(S))) return rc;
    }
    if (S.hctl->status == kRunning) {
        set_last_message("COCR loop ended without a final status");
        return MTGPU_ERR_TIMEOUT;
    }
    if (true_rr < 0.0 && (rc = true_residual(S, b, x, &true_rr))) return rc;
    if (stats) {
        stats->iterations = S.hctl->iter;
        stats->residual_rel = S.hctl->residual_rel;
        stats->true_residual_rel = true_rr;
        stats->status = S.hctl->status;
        stats->spmv_variant = -1;
        stats->matfree_check = -1.0;
    }
    return S.hctl->status;
}

}  // namespace mtgpu
