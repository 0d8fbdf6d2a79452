// Folded preconditioner  M^{-1} = D_A + G^T D_S G  on the device.
//
// G is the discrete gradient restricted to the interior nodes of conductive
// cells, with -1/2 for an edge's first node and +1/2 for its second
// (Code/COCR_FP/FoldedPreconditioner.cpp:68-259), D_A = diag(A)^{-1} and
// D_S = diag(G A G^T)^{-1} (FoldedPreconditioner.cpp:473-574).  The apply
// (FoldedPreconditioner.cpp:578-630) is a node gather followed by an edge
// gather; the COCR loop fuses both into its own kernels, the generic form
// here serves the set-up stages and the stand-alone entry point.
#include "mtgpu_internal.cuh"

#include <climits>

namespace mtgpu {

void Folded::release()
{
    dev_free(d_gp); dev_free(d_gj); dev_free(d_gv);
    dev_free(d_tp); dev_free(d_tj); dev_free(d_tv); dev_free(d_tn);
    dev_free(d_da); dev_free(d_ds); dev_free(d_h);
    n = m = 0;
}

int folded_build_g(const mtgpu_mesh_desc &mesh, Folded &P, cudaStream_t st)
{
    P.release();
    const int ne = mesh.n_edges_c, nn = mesh.n_nodes_c;
    MTGPU_CHECK_ARG(ne > 0 && nn > 0, "empty mesh");
    std::vector<char> in_sigma(nn, 0);
    for (int c = 0; c < mesh.kpar; c++) {
        if (!(mesh.sigma3d[mesh.nvkat[c]] > 0.0)) continue;
        for (int j = 0; j < 8; j++) {
            const int v = mesh.nver14[(size_t)c * mesh.nver_stride + j];
            if (v >= 0 && v < nn && !mesh.is_node_bound[v]) in_sigma[v] = 1;
        }
    }
    std::vector<int> renum(nn, -1);
    int m = 0;
    for (int v = 0; v < nn; v++)
        if (in_sigma[v]) renum[v] = m++;
    // G^T rows: the edge's first node (-1/2) then its second (+1/2); nodes
    // beyond n_nodes_c are expanded through the T-matrix rows ig_t/jg_t/gg_t
    std::vector<int> tp(ne + 1, 0), tj;
    std::vector<double> tv;
    std::vector<int2> tn(ne, make_int2(-1, -1));
    bool compact = true;
    tj.reserve((size_t)ne * 2);
    tv.reserve((size_t)ne * 2);
    for (int e = 0; e < ne; e++) {
        for (int k = 0; k < 2; k++) {
            const int v = mesh.edges2[2 * e + k];
            const double sgn = k == 0 ? -0.5 : 0.5;
            if (v < nn) {
                if (v >= 0 && in_sigma[v]) {
                    tj.push_back(renum[v]);
                    tv.push_back(sgn);
                    (k == 0 ? tn[e].x : tn[e].y) = renum[v];
                }
            } else {
                compact = false;
                for (int t = mesh.ig_t[v]; t < mesh.ig_t[v + 1]; t++)
                    if (in_sigma[mesh.jg_t[t]]) {
                        tj.push_back(renum[mesh.jg_t[t]]);
                        tv.push_back(sgn * mesh.gg_t[t]);
                    }
            }
        }
        tp[e + 1] = (int)tj.size();
    }
    const int nnz = tp[ne];
    std::vector<int> gp(m + 1, 0), gj(nnz > 0 ? nnz : 1), fill;
    std::vector<double> gv(nnz > 0 ? nnz : 1);
    for (int t = 0; t < nnz; t++) gp[tj[t] + 1]++;
    for (int i = 0; i < m; i++) gp[i + 1] += gp[i];
    fill.assign(gp.begin(), gp.end() - 1);
    for (int e = 0; e < ne; e++)
        for (int t = tp[e]; t < tp[e + 1]; t++) {
            const int r = tj[t];
            gj[fill[r]] = e;
            gv[fill[r]] = tv[t];
            fill[r]++;
        }
    P.n = ne;
    P.m = m;
    int rc;
    if ((rc = dev_alloc(&P.d_gp, m + 1)) || (rc = dev_alloc(&P.d_gj, nnz)) ||
        (rc = dev_alloc(&P.d_gv, nnz)) || (rc = dev_alloc(&P.d_tp, ne + 1)) ||
        (rc = dev_alloc(&P.d_tj, nnz)) || (rc = dev_alloc(&P.d_tv, nnz)) ||
        (rc = dev_alloc(&P.d_da, ne)) || (rc = dev_alloc(&P.d_ds, m)) ||
        (rc = dev_alloc(&P.d_h, m)))
        return rc;
    MTGPU_TRY(cudaMemcpyAsync(P.d_gp, gp.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice, st));
    if (nnz > 0) {
        MTGPU_TRY(cudaMemcpyAsync(P.d_gj, gj.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
        MTGPU_TRY(cudaMemcpyAsync(P.d_gv, gv.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
        MTGPU_TRY(cudaMemcpyAsync(P.d_tj, tj.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
        MTGPU_TRY(cudaMemcpyAsync(P.d_tv, tv.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
    }
    MTGPU_TRY(cudaMemcpyAsync(P.d_tp, tp.data(), sizeof(int) * (ne + 1), cudaMemcpyHostToDevice, st));
    if (compact) {
        if ((rc = dev_alloc(&P.d_tn, ne))) return rc;
        MTGPU_TRY(cudaMemcpyAsync(P.d_tn, tn.data(), sizeof(int2) * ne, cudaMemcpyHostToDevice, st));
    }
    // the host vectors go out of scope: wait for the copies
    MTGPU_TRY(cudaStreamSynchronize(st));
    return MTGPU_OK;
}

// ------------------------------------------------ G on the device
namespace {

// nodes of conductive cells that are not Dirichlet get a G row
__global__ void k_g_mark(int kpar, const int *__restrict__ nver, int stride,
                         const int *__restrict__ nvkat, const double *__restrict__ sigflag, int nmat,
                         int nn, const unsigned char *__restrict__ bnode, int *in_sig)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kpar) return;
    const int mat = nvkat[c];
    if (mat < 0 || mat >= nmat || !(sigflag[mat] > 0.0)) return;
    for (int j = 0; j < 8; j++) {
        const int v = nver[(size_t)c * stride + j];
        if (v >= 0 && v < nn && !bnode[v]) in_sig[v] = 1;
    }
}

// per edge its two nodes' G rows (-1 where none), the G^T row length and
// the G row lengths; *beyond counts edges with a node past nn
__global__ void k_g_edges(int ne, const int *__restrict__ edges, int nn, const int *__restrict__ in_sig,
                          const int *__restrict__ renum, int2 *tn, int *cnt_t, int *deg, int *beyond)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int r[2];
    for (int k = 0; k < 2; k++) {
        const int v = edges[2 * e + k];
        if (v >= nn) atomicAdd(beyond, 1);
        r[k] = v >= 0 && v < nn && in_sig[v] ? renum[v] : -1;
    }
    tn[e] = make_int2(r[0], r[1]);
    cnt_t[e] = (r[0] >= 0) + (r[1] >= 0);
    if (r[0] >= 0) atomicAdd(&deg[r[0]], 1);
    if (r[1] >= 0) atomicAdd(&deg[r[1]], 1);
}

// G^T rows in place (first node -1/2, then second +1/2); G entries at
// claimed positions of their rows (sorted afterwards)
__global__ void k_g_fill(int ne, const int2 *__restrict__ tn, const int *__restrict__ tp,
                         const int *__restrict__ gp, int *fill, int *tj, double *tv, int *gj,
                         double *gv)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int2 r = tn[e];
    int t = tp[e];
    const int rr[2] = {r.x, r.y};
    for (int k = 0; k < 2; k++) {
        if (rr[k] < 0) continue;
        const double g = k == 0 ? -0.5 : 0.5;
        tj[t] = rr[k];
        tv[t] = g;
        t++;
        const int q = gp[rr[k]] + atomicAdd(&fill[rr[k]], 1);
        gj[q] = e;
        gv[q] = g;
    }
}

// every G row by increasing edge (the order of the host construction)
__global__ void k_g_sort(int m, const int *__restrict__ gp, int *gj, double *gv)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m) return;
    const int b = gp[v], e = gp[v + 1];
    for (int i = b + 1; i < e; i++) {
        const int kj = gj[i];
        const double kv = gv[i];
        int j = i - 1;
        while (j >= b && gj[j] > kj) {
            gj[j + 1] = gj[j];
            gv[j + 1] = gv[j];
            j--;
        }
        gj[j + 1] = kj;
        gv[j + 1] = kv;
    }
}

__global__ void k_int_to_flag(int n, const int *__restrict__ in, unsigned char *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i] != 0;
}

// entries of an uploaded mesh description: bad[0] negative edge nodes,
// bad[1] edge nodes beyond nn (T-matrix nodes), bad[2] negative cell nodes
__global__ void k_check_mesh(int ne, int nn, const int *__restrict__ edges, int kpar,
                             const int *__restrict__ nver, int stride, int *bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ne) {
        const int a = edges[2 * i], b = edges[2 * i + 1];
        if (a < 0 || b < 0) atomicAdd(&bad[0], 1);
        if (a >= nn || b >= nn) atomicAdd(&bad[1], 1);
    }
    if (i < kpar) {
        int neg = 0;
        for (int j = 0; j < 8; j++) neg |= nver[(size_t)i * stride + j] < 0;
        if (neg) atomicAdd(&bad[2], 1);
    }
}

}  // namespace

int folded_build_g_device(const DevMesh &dm, Folded &P, cudaStream_t st, bool *conforming)
{
    P.release();
    *conforming = true;
    const int ne = dm.nb, nn = dm.nn;
    MTGPU_CHECK_ARG(ne > 0 && nn > 0, "empty mesh");
    MTGPU_CHECK_ARG(dm.nver && dm.nvkat && dm.edges && dm.sigflag && dm.bnode, "mesh tables missing");
    int *in_sig = nullptr, *renum = nullptr, *cnt_t = nullptr, *deg = nullptr, *fill = nullptr,
        *beyond = nullptr;
    auto done = [&](int code) {
        dev_free(in_sig); dev_free(renum); dev_free(cnt_t); dev_free(deg); dev_free(fill);
        dev_free(beyond);
        if (code != MTGPU_OK || !*conforming) P.release();
        return code;
    };
    int rc;
    if ((rc = dev_alloc(&in_sig, nn)) || (rc = dev_alloc(&renum, (size_t)nn + 1)) ||
        (rc = dev_alloc(&beyond, 1)))
        return done(rc);
    MTGPU_TRY(cudaMemsetAsync(in_sig, 0, sizeof(int) * nn, st));
    MTGPU_TRY(cudaMemsetAsync(beyond, 0, sizeof(int), st));
    if (dm.kpar > 0)
        k_g_mark<<<ceil_div(dm.kpar, kThreads), kThreads, 0, st>>>(dm.kpar, dm.nver, dm.nver_stride,
                                                                  dm.nvkat, dm.sigflag, dm.nmat, nn,
                                                                  dm.bnode, in_sig);
    note_launches(1);
    long long m64 = 0;
    if ((rc = dev_exclusive_scan(in_sig, nn, renum, &m64, st))) return done(rc);
    const int m = (int)m64;
    if ((rc = dev_alloc(&cnt_t, ne)) || (rc = dev_alloc(&deg, std::max(m, 1))) ||
        (rc = dev_alloc(&fill, std::max(m, 1))) || (rc = dev_alloc(&P.d_tn, ne)) ||
        (rc = dev_alloc(&P.d_tp, (size_t)ne + 1)) || (rc = dev_alloc(&P.d_gp, (size_t)m + 1)))
        return done(rc);
    MTGPU_TRY(cudaMemsetAsync(deg, 0, sizeof(int) * std::max(m, 1), st));
    MTGPU_TRY(cudaMemsetAsync(fill, 0, sizeof(int) * std::max(m, 1), st));
    k_g_edges<<<ceil_div(ne, kThreads), kThreads, 0, st>>>(ne, dm.edges, nn, in_sig, renum, P.d_tn,
                                                          cnt_t, deg, beyond);
    note_launches(1);
    int nbeyond = 0;
    MTGPU_TRY(cudaMemcpyAsync(&nbeyond, beyond, sizeof(int), cudaMemcpyDeviceToHost, st));
    MTGPU_TRY(cudaStreamSynchronize(st));
    if (nbeyond > 0) {
        *conforming = false;
        return done(MTGPU_OK);
    }
    long long nnz = 0, nnz_g = 0;
    if ((rc = dev_exclusive_scan(cnt_t, ne, P.d_tp, &nnz, st)) ||
        (rc = dev_exclusive_scan(deg, m, P.d_gp, &nnz_g, st)))
        return done(rc);
    MTGPU_CHECK_ARG(nnz == nnz_g, "G and G^T entry counts differ");
    if ((rc = dev_alloc(&P.d_tj, nnz)) || (rc = dev_alloc(&P.d_tv, nnz)) ||
        (rc = dev_alloc(&P.d_gj, nnz)) || (rc = dev_alloc(&P.d_gv, nnz)) ||
        (rc = dev_alloc(&P.d_da, ne)) || (rc = dev_alloc(&P.d_ds, m)) || (rc = dev_alloc(&P.d_h, m)))
        return done(rc);
    k_g_fill<<<ceil_div(ne, kThreads), kThreads, 0, st>>>(ne, P.d_tn, P.d_tp, P.d_gp, fill, P.d_tj,
                                                         P.d_tv, P.d_gj, P.d_gv);
    if (m > 0) k_g_sort<<<ceil_div(m, kThreads), kThreads, 0, st>>>(m, P.d_gp, P.d_gj, P.d_gv);
    note_launches(2);
    MTGPU_TRY(cudaGetLastError());
    P.n = ne;
    P.m = m;
    return done(MTGPU_OK);
}

int folded_build_g_auto(const mtgpu_mesh_desc &mesh, const DevMesh *dm, Folded &P, cudaStream_t st)
{
    DevMeshUpload dmu;
    int rc;
    if (!dm) {
        if ((rc = dmu.upload(mesh, nullptr, st))) return rc;
        dm = &dmu.view;
    }
    bool conforming = false;
    if ((rc = folded_build_g_device(*dm, P, st, &conforming))) return rc;
    return conforming ? MTGPU_OK : folded_build_g(mesh, P, st);
}

void DevMeshUpload::release()
{
    dev_free(nver); dev_free(nvkat); dev_free(edges); dev_free(xyz); dev_free(sigflag);
    dev_free(bnode);
    view = DevMesh{};
}

int DevMeshUpload::upload(const mtgpu_mesh_desc &m, const double *xyz_host, cudaStream_t st)
{
    release();
    int nmat = 0;
    for (int c = 0; c < m.kpar; c++) nmat = std::max(nmat, m.nvkat[c] + 1);
    nmat = std::max(nmat, 1);
    int *bound_i = nullptr;
    int rc;
    if ((rc = dev_alloc(&nver, (size_t)m.kpar * m.nver_stride)) ||
        (rc = dev_alloc(&nvkat, (size_t)m.kpar)) || (rc = dev_alloc(&edges, (size_t)m.n_edges_c * 2)) ||
        (rc = dev_alloc(&sigflag, (size_t)nmat)) || (rc = dev_alloc(&bnode, (size_t)m.n_nodes_c)) ||
        (rc = dev_alloc(&bound_i, (size_t)m.n_nodes_c)) ||
        (xyz_host && (rc = dev_alloc(&xyz, (size_t)m.n_nodes_c * 3)))) {
        dev_free(bound_i);
        return rc;
    }
    cudaError_t e = cudaSuccess;
    auto up = [&](void *d, const void *h, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
    };
    up(nver, m.nver14, sizeof(int) * (size_t)m.kpar * m.nver_stride);
    up(nvkat, m.nvkat, sizeof(int) * (size_t)m.kpar);
    up(edges, m.edges2, sizeof(int) * (size_t)m.n_edges_c * 2);
    up(sigflag, m.sigma3d, sizeof(double) * (size_t)nmat);
    up(bound_i, m.is_node_bound, sizeof(int) * (size_t)m.n_nodes_c);
    if (xyz_host) up(xyz, xyz_host, sizeof(double) * (size_t)m.n_nodes_c * 3);
    // the entries the host validation of a mesh description checks
    int *d_bad = nullptr, bad[3] = {0, 0, 0};
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_bad, sizeof(int) * 3);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(int) * 3, st);
    if (e == cudaSuccess) {
        k_int_to_flag<<<ceil_div(m.n_nodes_c, kThreads), kThreads, 0, st>>>(m.n_nodes_c, bound_i, bnode);
        k_check_mesh<<<ceil_div(std::max(m.n_edges_c, m.kpar), kThreads), kThreads, 0, st>>>(
            m.n_edges_c, m.n_nodes_c, edges, m.kpar, nver, m.nver_stride, d_bad);
        note_launches(2);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, st);
    // the host arrays are the caller's: the copies must end before it returns
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dev_free(bound_i);
    dev_free(d_bad);
    if (e != cudaSuccess) {
        set_last_error(e, "mesh upload", __FILE__, __LINE__);
        return MTGPU_ERR_CUDA;
    }
    MTGPU_CHECK_ARG(bad[0] == 0, "negative node in edges");
    MTGPU_CHECK_ARG(bad[1] == 0 || (m.ig_t && m.jg_t && m.gg_t),
                    "edge node beyond n_nodes_c without T-matrix");
    MTGPU_CHECK_ARG(bad[2] == 0, "bad nver");
    view.kpar = m.kpar;
    view.nb = m.n_edges_c;
    view.nn = m.n_nodes_c;
    view.nver_stride = m.nver_stride;
    view.nmat = nmat;
    view.xyz = xyz;
    view.nver = nver;
    view.nvkat = nvkat;
    view.edges = edges;
    view.sigflag = sigflag;
    view.bnode = bnode;
    return MTGPU_OK;
}

int DevMeshUpload::over_device(int kpar, int nb, int nn, int nver_stride, const double *d_xyz,
                               const int *d_nver, const int *d_nvkat, const int *d_edges,
                               const unsigned char *d_bnode, const double *sigflag_host, int nmat,
                               cudaStream_t st)
{
    release();
    nmat = std::max(nmat, 1);
    int rc = dev_alloc(&sigflag, (size_t)nmat);
    if (rc) return rc;
    MTGPU_TRY(cudaMemcpyAsync(sigflag, sigflag_host, sizeof(double) * nmat, cudaMemcpyHostToDevice, st));
    MTGPU_TRY(cudaStreamSynchronize(st));
    view.kpar = kpar;
    view.nb = nb;
    view.nn = nn;
    view.nver_stride = nver_stride;
    view.nmat = nmat;
    view.xyz = d_xyz;
    view.nver = d_nver;
    view.nvkat = d_nvkat;
    view.edges = d_edges;
    view.sigflag = sigflag;
    view.bnode = d_bnode;
    return MTGPU_OK;
}

namespace {

__device__ inline long long slot(const long long *p, int row, int k)
{
    return p[row / kSlice] + (long long)k * kSlice + (row % kSlice);
}

__global__ void k_diag_a(int nb, const long long *pc, const int *col_c, const double2 *val_c,
                         const int *diag_slot, double2 *da)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const int k = diag_slot[i];
    const double2 d = k >= 0 ? val_c[slot(pc, i, k)] : make_double2(0.0, 0.0);
    da[i] = cdiv(make_double2(1.0, 0.0), d);
}

// D_S[v] = 1 / sum_{k,c in row v of G} g_k g_c A[k][c].
// Re diag(G A G^T) is a cancellation (the curl-curl part annihilates
// gradients) and in the air it is not small next to the tiny imaginary
// part, so D_S there depends on the summation order.  This kernel therefore
// adds in the reference's order — row k of A by increasing column, complex
// and real entries merged (FoldedPreconditioner.cpp:518-556 over the rows
// of From2x2ToCSR2x2_2) — with unfused multiply and add.
__global__ void k_diag_s(int m, const int *gp, const int *gj, const double *gv,
                         const int *nc_row, const int *nr_row, const long long *pc,
                         const long long *pr, const int *col_c, const double2 *val_c,
                         const int *col_r, const double *val_r, double2 *ds)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m) return;
    const int b = gp[v], e = gp[v + 1];
    double sr = 0.0, si = 0.0;
    for (int j = b; j < e; j++) {
        const int k = gj[j];
        const double gk = gv[j];
        const int nc = nc_row[k], nr = nr_row[k];
        double tr = 0.0, ti = 0.0;
        int qc = 0, qr = 0;
        while (qc < nc || qr < nr) {
            const int cc = qc < nc ? col_c[slot(pc, k, qc)] : INT_MAX;
            const int cr = qr < nr ? col_r[slot(pr, k, qr)] : INT_MAX;
            double ar, ai;
            int c;
            if (cc < cr) {
                const double2 a = val_c[slot(pc, k, qc++)];
                ar = a.x;
                ai = a.y;
                c = cc;
            } else {
                ar = val_r[slot(pr, k, qr++)];
                ai = 0.0;
                c = cr;
            }
            for (int u = b; u < e; u++)
                if (gj[u] == c) {
                    tr = __dadd_rn(tr, __dmul_rn(ar, gv[u]));
                    ti = __dadd_rn(ti, __dmul_rn(ai, gv[u]));
                }
        }
        sr = __dadd_rn(sr, __dmul_rn(tr, gk));
        si = __dadd_rn(si, __dmul_rn(ti, gk));
    }
    ds[v] = cdiv(make_double2(1.0, 0.0), make_double2(sr, si));
}

__global__ void k_node(int m, const int *__restrict__ gp, const int *__restrict__ gj,
                       const double *__restrict__ gv, const double2 *__restrict__ ds,
                       const double2 *__restrict__ x, double2 *__restrict__ h)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m) return;
    double hr = 0.0, hi = 0.0;
    for (int j = gp[v]; j < gp[v + 1]; j++) {
        const double2 xv = x[gj[j]];
        hr += gv[j] * xv.x;
        hi += gv[j] * xv.y;
    }
    h[v] = cmul(make_double2(hr, hi), ds[v]);
}

__global__ void k_edge(int n, const int *__restrict__ tp, const int *__restrict__ tj,
                       const double *__restrict__ tv, const double2 *__restrict__ da,
                       const double2 *__restrict__ h, const double2 *__restrict__ x,
                       double2 *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 acc = cmul(x[i], da[i]);
    for (int j = tp[i]; j < tp[i + 1]; j++) {
        const double2 hv = h[tj[j]];
        acc.x += tv[j] * hv.x;
        acc.y += tv[j] * hv.y;
    }
    y[i] = acc;
}

}  // namespace

int folded_build_diag(const SellMatrix &A, Folded &P, cudaStream_t st)
{
    k_diag_a<<<ceil_div(A.nb, kThreads), kThreads, 0, st>>>(A.nb, A.d_pc, A.d_col_c, A.d_val_c,
                                                            A.d_diag_slot, P.d_da);
    if (P.m > 0)
        k_diag_s<<<ceil_div(P.m, 128), 128, 0, st>>>(P.m, P.d_gp, P.d_gj, P.d_gv, A.d_nc, A.d_nr,
                                                     A.d_pc, A.d_pr, A.d_col_c, A.d_val_c,
                                                     A.d_col_r, A.d_val_r, P.d_ds);
    MTGPU_TRY(cudaGetLastError());
    return MTGPU_OK;
}

void folded_apply(const Folded &P, const double2 *x, double2 *y, cudaStream_t st)
{
    if (P.m > 0)
        k_node<<<ceil_div(P.m, kThreads), kThreads, 0, st>>>(P.m, P.d_gp, P.d_gj, P.d_gv, P.d_ds,
                                                             x, P.d_h);
    k_edge<<<ceil_div(P.n, kThreads), kThreads, 0, st>>>(P.n, P.d_tp, P.d_tj, P.d_tv, P.d_da,
                                                         P.d_h, x, y);
}

}  // namespace mtgpu
