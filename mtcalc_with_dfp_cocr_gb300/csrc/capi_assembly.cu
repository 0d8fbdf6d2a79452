// extern "C" entry points of the device assembly (include/mtgpu.h).
#include "assemble.cuh"

#include <cmath>

using namespace mtgpu;

namespace {
constexpr double kTwoPi = 2.0 * 3.1415926535897932384626433832795;   // BuildMatrix/stdafx.h:32

template <class T>
int upload_vec(T **d, const T *h, size_t n, cudaStream_t st)
{
    int rc = dev_alloc(d, n);
    if (rc) return rc;
    if (n) MTGPU_TRY(cudaMemcpyAsync(*d, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
    return MTGPU_OK;
}
}  // namespace

extern "C" {

int mtgpu_assembly_create(const mtgpu_fem_mesh *mesh, mtgpu_assembly **out)
{
    MTGPU_CHECK_ARG(mesh && out, "null argument");
    *out = nullptr;
    auto *a = new mtgpu_assembly_s();
    cudaError_t e = cudaStreamCreateWithFlags(&a->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete a;
        set_last_error(e, "cudaStreamCreateWithFlags", __FILE__, __LINE__);
        return MTGPU_ERR_CUDA;
    }
    int rc = param_assemble(*mesh, a->P, a->st);
    if (rc) {
        mtgpu_assembly_destroy(a);
        return rc;
    }
    const mtgpu_fem_mesh &m = *mesh;
    a->nver_stride = m.nver_stride;
    a->nver.assign(m.nver, m.nver + (size_t)m.kpar * m.nver_stride);
    a->nvkat.assign(m.nvkat, m.nvkat + m.kpar);
    a->xyz.assign(m.xyz, m.xyz + (size_t)3 * m.kuzlov);
    a->edges.assign(m.edges, m.edges + (size_t)2 * m.nb);
    a->bound.assign(m.kuzlov, 0);
    for (int i = 0; i < m.n_bound; i++) a->bound[m.bound_nodes[i]] = 1;
    a->sigflag.resize(m.n_materials);
    for (int i = 0; i < m.n_materials; i++) a->sigflag[i] = m.sigma[i] == 0.0 ? 0.0 : 1.0;
    a->ig_t.assign(m.kuzlov + 1, 0);
    *out = a;
    return MTGPU_OK;
}

int mtgpu_assembly_create_regular(int nx, int ny, int nz, const double *x, const double *y,
                                  const double *z, const int *cell_material, int n_materials,
                                  const double *mu, const double *sigma, const double *sigma0,
                                  mtgpu_assembly **out)
{
    MTGPU_CHECK_ARG(out != nullptr, "null argument");
    *out = nullptr;
    auto *a = new mtgpu_assembly_s();
    cudaError_t e = cudaStreamCreateWithFlags(&a->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete a;
        set_last_error(e, "cudaStreamCreateWithFlags", __FILE__, __LINE__);
        return MTGPU_ERR_CUDA;
    }
    int rc = param_assemble_regular(nx, ny, nz, x, y, z, cell_material, n_materials, mu, sigma,
                                    sigma0, a->P, a->st);
    if (rc) {
        mtgpu_assembly_destroy(a);
        return rc;
    }
    // host copies for the host-side set-up (preconditioner pattern, matrix-free
    // tables, receiver location): the device's own tables, read back once
    const ParamMatrix &P = a->P;
    a->nver_stride = 8;
    a->nver.resize((size_t)P.kpar * 8);
    a->xyz.resize((size_t)P.kuzlov * 3);
    a->edges.resize((size_t)P.nb * 2);
    a->nvkat.assign(cell_material, cell_material + P.kpar);
    auto dn = [&](void *h, const void *d, size_t bytes) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, a->st);
    };
    dn(a->nver.data(), P.d_nver, sizeof(int) * a->nver.size());
    dn(a->xyz.data(), P.d_xyz, sizeof(double) * a->xyz.size());
    dn(a->edges.data(), P.d_edges, sizeof(int) * a->edges.size());
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->st);
    if (e != cudaSuccess) {
        set_last_error(e, "mtgpu_assembly_create_regular", __FILE__, __LINE__);
        mtgpu_assembly_destroy(a);
        return MTGPU_ERR_CUDA;
    }
    a->bound.assign(P.kuzlov, 0);
    for (int k = 0, n = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++, n++)
                a->bound[n] = i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1;
    a->sigflag.resize(n_materials);
    for (int i = 0; i < n_materials; i++) a->sigflag[i] = sigma[i] == 0.0 ? 0.0 : 1.0;
    a->ig_t.assign(P.kuzlov + 1, 0);
    *out = a;
    return MTGPU_OK;
}

void mtgpu_assembly_destroy(mtgpu_assembly *a)
{
    if (!a) return;
    if (a->st) cudaStreamSynchronize(a->st);
    a->P.release();
    if (a->st) cudaStreamDestroy(a->st);
    delete a;
}

int mtgpu_assembly_check_preconditioner(mtgpu_assembly *a, int *equal)
{
    MTGPU_CHECK_ARG(a && equal, "null argument");
    *equal = 0;
    const ParamMatrix &P = a->P;
    const mtgpu_mesh_desc mesh{P.kpar, P.nb, P.kuzlov, a->nvkat.data(), a->nver.data(),
                               a->sigflag.data(), a->edges.data(), a->ig_t.data(), a->ig_t.data(),
                               nullptr, a->bound.data(), a->nver_stride};
    Folded H, D;
    DevMeshUpload dmu;
    bool conforming = false;
    int rc;
    if ((rc = folded_build_g(mesh, H, a->st)) ||
        (rc = dmu.over_device(P.kpar, P.nb, P.kuzlov, P.nver_stride, P.d_xyz, P.d_nver, P.d_nvkat,
                              P.d_edges, P.d_bnode, a->sigflag.data(), (int)a->sigflag.size(),
                              a->st)) ||
        (rc = folded_build_g_device(dmu.view, D, a->st, &conforming)))
        return rc;
    if (!conforming || H.n != D.n || H.m != D.m || !H.d_tn || !D.d_tn) return MTGPU_OK;
    const int n = H.n, m = H.m;
    int nnz_h = 0, nnz_d = 0;
    MTGPU_TRY(cudaMemcpyAsync(&nnz_h, H.d_gp + m, sizeof(int), cudaMemcpyDeviceToHost, a->st));
    MTGPU_TRY(cudaMemcpyAsync(&nnz_d, D.d_gp + m, sizeof(int), cudaMemcpyDeviceToHost, a->st));
    MTGPU_TRY(cudaStreamSynchronize(a->st));
    if (nnz_h != nnz_d) return MTGPU_OK;
    bool same = true;
    auto cmp = [&](const void *dh, const void *dd, size_t bytes) -> int {
        if (!same || bytes == 0) return MTGPU_OK;
        std::vector<unsigned char> x(bytes), y(bytes);
        MTGPU_TRY(cudaMemcpyAsync(x.data(), dh, bytes, cudaMemcpyDeviceToHost, a->st));
        MTGPU_TRY(cudaMemcpyAsync(y.data(), dd, bytes, cudaMemcpyDeviceToHost, a->st));
        MTGPU_TRY(cudaStreamSynchronize(a->st));
        same = x == y;
        return MTGPU_OK;
    };
    const size_t nz = (size_t)nnz_h;
    if ((rc = cmp(H.d_gp, D.d_gp, sizeof(int) * ((size_t)m + 1))) ||
        (rc = cmp(H.d_gj, D.d_gj, sizeof(int) * nz)) || (rc = cmp(H.d_gv, D.d_gv, sizeof(double) * nz)) ||
        (rc = cmp(H.d_tp, D.d_tp, sizeof(int) * ((size_t)n + 1))) ||
        (rc = cmp(H.d_tj, D.d_tj, sizeof(int) * nz)) || (rc = cmp(H.d_tv, D.d_tv, sizeof(double) * nz)) ||
        (rc = cmp(H.d_tn, D.d_tn, sizeof(int2) * (size_t)n)))
        return rc;
    *equal = same ? 1 : 0;
    return MTGPU_OK;
}

int mtgpu_assembly_info(const mtgpu_assembly *a, long long *nnz_complex, long long *nnz_real,
                        int *nnz_lower, long long *gg_len)
{
    MTGPU_CHECK_ARG(a != nullptr, "null assembly");
    const ParamMatrix &P = a->P;
    if (nnz_complex) *nnz_complex = P.nnz_c;
    if (nnz_real) *nnz_real = P.nnz_r;
    // the pattern is symmetric with every diagonal present
    if (nnz_lower) *nnz_lower = (int)((P.nnz_c - P.nb) / 2 + P.nnz_r / 2);
    if (gg_len) *gg_len = (P.nnz_c - P.nb) + P.nnz_r / 2;
    return MTGPU_OK;
}

int mtgpu_assembly_rhs(mtgpu_assembly *a, int S, const double *nu, const int *alfa, int n1d,
                       const double *z1d, const double *usin, const double *ucos, double *d_rhs)
{
    MTGPU_CHECK_ARG(a && nu && alfa && z1d && usin && ucos && d_rhs, "null argument");
    MTGPU_CHECK_ARG(S > 0 && n1d >= 2, "bad sizes");
    for (int i = 0; i + 1 < n1d; i++) MTGPU_CHECK_ARG(z1d[i] <= z1d[i + 1], "z1d must ascend");
    std::vector<double> om(S);
    for (int k = 0; k < S; k++) om[k] = kTwoPi * nu[k];
    double *d_om = nullptr, *d_z = nullptr, *d_us = nullptr, *d_uc = nullptr;
    int *d_al = nullptr;
    int rc;
    MTGPU_TRY(cudaStreamSynchronize(cudaStreamLegacy));
    if (!(rc = upload_vec(&d_om, om.data(), S, a->st)) && !(rc = upload_vec(&d_al, alfa, S, a->st)) &&
        !(rc = upload_vec(&d_z, z1d, n1d, a->st)) &&
        !(rc = upload_vec(&d_us, usin, (size_t)S * n1d, a->st)) &&
        !(rc = upload_vec(&d_uc, ucos, (size_t)S * n1d, a->st))) {
        rc = param_rhs(a->P, S, d_om, d_al, n1d, d_z, d_us, d_uc, (double2 *)d_rhs, a->P.nb, 0, a->st);
        cudaError_t e = cudaStreamSynchronize(a->st);
        if (!rc && e != cudaSuccess) {
            set_last_error(e, "mtgpu_assembly_rhs", __FILE__, __LINE__);
            rc = MTGPU_ERR_CUDA;
        }
    }
    dev_free(d_om); dev_free(d_al); dev_free(d_z); dev_free(d_us); dev_free(d_uc);
    return rc;
}

int mtgpu_assembly_block2x2(mtgpu_assembly *a, double nu, int alfa, int n1d, const double *z1d,
                            const double *usin, const double *ucos, int *ig, int *jg, int *idi,
                            int *ijg, double *di, double *gg, double *pr)
{
    MTGPU_CHECK_ARG(a && ig && jg && idi && ijg && di && gg && pr, "null argument");
    const int nb = a->P.nb;
    Block2x2Dev B;
    int rc = param_to_block2x2(a->P, kTwoPi * nu, B, a->st);
    double *d_rhs = nullptr;
    if (!rc) rc = dev_alloc(&d_rhs, (size_t)2 * nb);
    if (!rc) rc = mtgpu_assembly_rhs(a, 1, &nu, &alfa, n1d, z1d, usin, ucos, d_rhs);
    if (!rc) {
        cudaError_t e = cudaSuccess;
        auto cp = [&](void *dst, const void *src, size_t bytes) {
            if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, a->st);
        };
        cp(ig, B.ig, sizeof(int) * (nb + 1));
        cp(jg, B.jg, sizeof(int) * B.nnz);
        cp(idi, B.idi, sizeof(int) * (nb + 1));
        cp(ijg, B.ijg, sizeof(int) * (B.nnz + 1));
        cp(di, B.di, sizeof(double) * 2 * nb);
        cp(gg, B.gg, sizeof(double) * B.gg_len);
        cp(pr, d_rhs, sizeof(double) * 2 * nb);
        if (e == cudaSuccess) e = cudaStreamSynchronize(a->st);
        if (e != cudaSuccess) {
            set_last_error(e, "mtgpu_assembly_block2x2", __FILE__, __LINE__);
            rc = MTGPU_ERR_CUDA;
        }
    }
    dev_free(d_rhs);
    B.release();
    return rc;
}

int mtgpu_cocr_create_from_assembly(mtgpu_assembly *a, double nu, void *stream, mtgpu_cocr **out)
{
    MTGPU_CHECK_ARG(a && out, "null argument");
    *out = nullptr;
    auto *c = new mtgpu_cocr_s();
    int rc = make_stream(c, stream);
    if (rc) {
        delete c;
        return rc;
    }
    CocrSolver &S = c->S;
    S.nb = a->P.nb;
    mtgpu_mesh_desc mesh{a->P.kpar, a->P.nb, a->P.kuzlov, a->nvkat.data(), a->nver.data(),
                         a->sigflag.data(), a->edges.data(), a->ig_t.data(), a->ig_t.data(),
                         nullptr, a->bound.data(), a->nver_stride};
    DevMeshUpload dmu;
    const ParamMatrix &P = a->P;
    if (!(rc = param_to_sell(a->P, kTwoPi * nu, S.A, S.st)) &&
        !(rc = dmu.over_device(P.kpar, P.nb, P.kuzlov, P.nver_stride, P.d_xyz, P.d_nver, P.d_nvkat,
                               P.d_edges, P.d_bnode, a->sigflag.data(), (int)a->sigflag.size(),
                               S.st)) &&
        !(rc = folded_build_g_auto(mesh, &dmu.view, S.P, S.st)) &&
        !(rc = folded_build_diag(S.A, S.P, S.st)) && !(rc = cocr_alloc(S))) {
        note_launches(2);
        cudaError_t e = cudaStreamSynchronize(S.st);
        if (e != cudaSuccess) {
            set_last_error(e, "mtgpu_cocr_create_from_assembly", __FILE__, __LINE__);
            rc = MTGPU_ERR_CUDA;
        }
    }
    if (rc) {
        mtgpu_cocr_destroy(c);
        return rc;
    }
    *out = c;
    return MTGPU_OK;
}

}  // extern "C"

// ------------------------------------------------------------ survey
#include "survey.cuh"

#include <memory>

// A survey: its systems, mesh by mesh, cut into batches (groups) of at most
// 32 systems of one mesh, each with its own stream and CUDA graph.  The
// systems' vectors are packed one after the other (system k at sys_off[k]
// doubles) in the caller's d_b / d_x.
struct mtgpu_survey_s {
    std::vector<std::unique_ptr<mtgpu::Survey>> groups;
    std::vector<int> g_first;                 // first system of every group
    std::vector<cudaStream_t> g_st;           // stream of every group (owned)
    std::vector<double> nu;                   // frequency of every system
    std::vector<mtgpu_assembly *> sys_asm;    // assembly of every system
    std::vector<long long> sys_off;           // [S + 1] offsets in doubles
    cudaStream_t user = nullptr;              // the caller's stream (NULL: legacy default)
};

extern "C" {

void mtgpu_survey_destroy(mtgpu_survey *s)
{
    if (!s) return;
    for (size_t g = 0; g < s->groups.size(); g++) {
        if (s->g_st[g]) cudaStreamSynchronize(s->g_st[g]);
        s->groups[g]->release();
        if (s->g_st[g]) cudaStreamDestroy(s->g_st[g]);
    }
    delete s;
}

int mtgpu_survey_create_multi(int nmesh, mtgpu_assembly *const *a, const int *S, const double *nu,
                              void *stream, mtgpu_survey **out)
{
    MTGPU_CHECK_ARG(a && S && nu && out && nmesh >= 1, "null argument");
    *out = nullptr;
    int total = 0;
    for (int m = 0; m < nmesh; m++) {
        MTGPU_CHECK_ARG(a[m] != nullptr, "null assembly");
        MTGPU_CHECK_ARG(S[m] >= 1, "every mesh needs at least one system");
        total += S[m];
    }
    MTGPU_CHECK_ARG(total <= MTGPU_SURVEY_MAX_SYSTEMS, "a survey holds at most "
                    "MTGPU_SURVEY_MAX_SYSTEMS (256) systems");
    for (int k = 0; k < total; k++) MTGPU_CHECK_ARG(nu[k] > 0.0, "frequencies must be positive");
    auto *s = new mtgpu_survey_s();
    s->user = (cudaStream_t)stream;
    s->nu.assign(nu, nu + total);
    s->sys_off.assign(1, 0);
    int k0 = 0;
    for (int m = 0; m < nmesh; m++) {
        mtgpu_assembly *am = a[m];
        mtgpu_mesh_desc mesh{am->P.kpar, am->P.nb, am->P.kuzlov, am->nvkat.data(), am->nver.data(),
                             am->sigflag.data(), am->edges.data(), am->ig_t.data(), am->ig_t.data(),
                             nullptr, am->bound.data(), am->nver_stride};
        for (int k = 0; k < S[m]; k++) {
            s->sys_asm.push_back(am);
            s->sys_off.push_back(s->sys_off.back() + 2LL * am->P.nb);
        }
        // batches of 32 systems, the last one smaller
        for (int f = 0; f < S[m]; f += 32) {
            const int n = std::min(32, S[m] - f);
            cudaStream_t st = nullptr;
            cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
            if (e != cudaSuccess) {
                mtgpu_survey_destroy(s);
                set_last_error(e, "cudaStreamCreateWithFlags", __FILE__, __LINE__);
                return MTGPU_ERR_CUDA;
            }
            s->groups.push_back(std::make_unique<mtgpu::Survey>());
            s->g_st.push_back(st);
            s->g_first.push_back(k0 + f);
            std::vector<double> om(n);
            for (int k = 0; k < n; k++) om[k] = kTwoPi * nu[k0 + f + k];
            int sp = 1;
            while (sp < n) sp <<= 1;
            const auto tu = am->tuned.find(sp);
            int rc = survey_setup(am->P, mesh, n, om.data(), *s->groups.back(), st, am,
                                  nullptr, tu != am->tuned.end() ? tu->second : -1);
            if (!rc && s->groups.back()->autotuned) am->tuned[sp] = s->groups.back()->ch;
            if (rc) {
                mtgpu_survey_destroy(s);
                return rc;
            }
        }
        k0 += S[m];
    }
    *out = s;
    return MTGPU_OK;
}

int mtgpu_survey_create(mtgpu_assembly *a, int S, const double *nu, void *stream,
                        mtgpu_survey **out)
{
    return mtgpu_survey_create_multi(1, &a, &S, nu, stream, out);
}

int mtgpu_survey_info(const mtgpu_survey *s, int *S, int *groups, long long *offsets)
{
    MTGPU_CHECK_ARG(s != nullptr, "null survey");
    if (S) *S = (int)s->nu.size();
    if (groups) *groups = (int)s->groups.size();
    if (offsets)
        for (size_t k = 0; k < s->sys_off.size(); k++) offsets[k] = s->sys_off[k];
    return MTGPU_OK;
}

int mtgpu_survey_solve(mtgpu_survey *s, const double *d_b, double *d_x, double eps, int maxiter,
                       int verify, mtgpu_survey_stats *stats)
{
    MTGPU_CHECK_ARG(s && d_b && d_x, "null argument");
    MTGPU_CHECK_ARG(eps > 0.0, "eps must be positive");
    MTGPU_TRY(cudaStreamSynchronize(cudaStreamLegacy));
    if (s->user) MTGPU_TRY(cudaStreamSynchronize(s->user));
    const double t0 = now_seconds();
    mtgpu_survey_stats local{};
    mtgpu_survey_stats *st = stats ? stats : &local;
    // every batch started, then launched and collected in turn, so that
    // their graphs run side by side on the GPU
    const size_t ng = s->groups.size();
    std::vector<SurveyRun> R(ng);
    int rc = MTGPU_OK;
    for (size_t g = 0; g < ng && !rc; g++) {
        const long long off = s->sys_off[s->g_first[g]];
        rc = survey_begin(*s->groups[g], (const double2 *)(d_b + off), (double2 *)(d_x + off), eps,
                          maxiter, verify, 16, R[g]);
    }
    for (bool busy = true; !rc && busy;) {
        busy = false;
        for (size_t g = 0; g < ng && !rc; g++) rc = survey_launch(*s->groups[g], R[g]);
        for (size_t g = 0; g < ng && !rc; g++) {
            rc = survey_collect(*s->groups[g], R[g]);
            busy |= !R[g].done;
        }
    }
    for (size_t g = 0; g < ng && !rc; g++) {
        const int r2 = survey_finish(*s->groups[g], R[g], st, s->g_first[g]);
        if (r2 <= MTGPU_ERR_ARG) rc = r2;
    }
    for (auto &r : R) r.release();
    if (rc <= MTGPU_ERR_ARG) {
        for (size_t g = 0; g < ng; g++) cudaStreamSynchronize(s->g_st[g]);
        return rc;
    }
    // systems the double-float iteration could not finish: FP64 COCR with the
    // iterations left.  A double-float solution within 100 eps of the target
    // is the FP64 iteration's start; a stalled one (far above: very low
    // frequencies, large errors in the air's gradient components, from which
    // the FP64 iteration does not recover) is discarded for x = 0.
    int worst = MTGPU_OK;
    const int S = (int)s->nu.size();
    cudaStream_t st0 = s->g_st[0];
    for (int k = 0; k < S; k++) {
        const int left = maxiter - st->iterations[k];
        const long long off = s->sys_off[k], n = s->sys_off[k + 1] - off;
        if (st->status[k] == MTGPU_MAXITER && left > 0) {
            mtgpu_cocr *c = nullptr;
            int r2 = mtgpu_cocr_create_from_assembly(s->sys_asm[k], s->nu[k], st0, &c);
            if (r2) return r2;
            mtgpu_solve_opts opts{verify, 0, 0};
            mtgpu_solve_stats s64{};
            const double tr = st->true_residual_rel[k];
            if (!(tr >= 0.0 && tr < 100.0 * eps))
                MTGPU_TRY(cudaMemsetAsync(d_x + off, 0, sizeof(double) * n, st0));
            MTGPU_TRY(cudaStreamSynchronize(st0));
            r2 = mtgpu_cocr_solve(c, d_b + off, d_x + off, eps, left, &opts, &s64);
            mtgpu_cocr_destroy(c);
            if (r2 <= MTGPU_ERR_ARG) return r2;
            st->status[k] = r2;
            st->fp64_iterations[k] = s64.iterations;
            st->true_residual_rel[k] = s64.true_residual_rel;
            st->residual_rel[k] = s64.residual_rel;
        }
        if (st->status[k] != MTGPU_OK && worst == MTGPU_OK) worst = st->status[k];
    }
    st->seconds = now_seconds() - t0;
    return worst;
}

int mtgpu_survey_tuning(const mtgpu_survey *s, int *variant, float *ms)
{
    MTGPU_CHECK_ARG(s != nullptr, "null survey");
    const mtgpu::Survey &V = *s->groups[0];
    if (variant) *variant = V.ch;
    if (ms)
        for (int i = 0; i < kSpmvVariants; i++) ms[i] = V.tune_ms[i];
    return MTGPU_OK;
}

int mtgpu_survey_preconditioner(const mtgpu_survey *s, int *fused, float *ms)
{
    MTGPU_CHECK_ARG(s != nullptr, "null survey");
    const mtgpu::Survey &V = *s->groups[0];
    if (fused) *fused = V.prec_tile ? 1 : 0;
    if (ms) {
        ms[0] = V.prec_ms[0];
        ms[1] = V.prec_ms[1];
    }
    return MTGPU_OK;
}

int mtgpu_survey_set_spmv_variant(mtgpu_survey *s, int variant)
{
    MTGPU_CHECK_ARG(s != nullptr, "null survey");
    for (auto &g : s->groups) {
        const int rc = survey_prepare_variant(*g, variant);
        if (rc) return rc;
    }
    for (auto &g : s->groups)
        MTGPU_CHECK_ARG(spmv_variant_available(*g, variant),
                        "unknown SpMV variant, or not available for this survey");
    for (auto &g : s->groups) {
        const int rc = survey_set_variant(*g, variant);
        if (rc) return rc;
    }
    return MTGPU_OK;
}

int mtgpu_survey_spmv_timed(mtgpu_survey *s, int reps, float *ms)
{
    MTGPU_CHECK_ARG(s && ms && reps > 0, "bad argument");
    return survey_spmv_timed(*s->groups[0], reps, ms);
}

int mtgpu_survey_spmv(mtgpu_survey *s, const double *d_x, double *d_y)
{
    MTGPU_CHECK_ARG(s && d_x && d_y, "null argument");
    MTGPU_TRY(cudaStreamSynchronize(cudaStreamLegacy));
    if (s->user) MTGPU_TRY(cudaStreamSynchronize(s->user));
    for (size_t g = 0; g < s->groups.size(); g++) {
        const long long off = s->sys_off[s->g_first[g]];
        const int rc = survey_spmv(*s->groups[g], (const double2 *)(d_x + off), (double2 *)(d_y + off));
        if (rc) return rc;
    }
    return MTGPU_OK;
}

}  // extern "C"
