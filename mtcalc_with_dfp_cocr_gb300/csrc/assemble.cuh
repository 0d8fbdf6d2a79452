// Device assembly: parametric matrix A(omega) = K + i omega M on a SELL-32
// pattern, per-system right-hand sides, and conversion to the reference's
// lower-triangle block format.
#pragma once
#include "mtgpu_internal.cuh"

#include <map>
#include <vector>

namespace mtgpu {

struct ParamMatrix {
    int nb = 0, kpar = 0, kuzlov = 0, n_materials = 0;
    int ed_stride = 12, nver_stride = 8;
    int nslices = 0;
    long long nnz_c = 0, nnz_r = 0, len_c = 0, len_r = 0;
    // pattern (same layout as SellMatrix)
    int *d_wc = nullptr, *d_wr = nullptr;
    long long *d_pc = nullptr, *d_pr = nullptr;
    int *d_nc = nullptr, *d_nr = nullptr;
    int *d_col_c = nullptr, *d_col_r = nullptr;
    // values: K on complex and real slots, M on complex slots
    double *d_kc = nullptr, *d_mc = nullptr, *d_kr = nullptr;
    // mesh on the device
    int *d_ec_ptr = nullptr, *d_ec_cell = nullptr;    // edge -> (cell << 4 | local edge)
    double *d_xyz = nullptr;
    int *d_nver = nullptr, *d_ed = nullptr, *d_edges = nullptr, *d_nvkat = nullptr;
    double *d_mu = nullptr, *d_sig = nullptr, *d_sig0 = nullptr;
    unsigned char *d_bedge = nullptr;                  // Dirichlet edges
    unsigned char *d_bnode = nullptr;                  // Dirichlet nodes
    void release();
};

struct Block2x2Dev {
    int nb = 0, nnz = 0;
    long long gg_len = 0;
    int *ig = nullptr, *jg = nullptr, *idi = nullptr, *ijg = nullptr;
    double *di = nullptr, *gg = nullptr;
    void release();
};

int param_assemble(const mtgpu_fem_mesh &m, ParamMatrix &P, cudaStream_t st);
// the device part: P's mesh tables and sizes set, bnode[kuzlov] the Dirichlet node flags
int param_build(ParamMatrix &P, const unsigned char *bnode, cudaStream_t st);
// a regular mesh from its node lines: every table generated on the device (regular_mesh.cu)
int param_assemble_regular(int nx, int ny, int nz, const double *x, const double *y,
                           const double *z, const int *cell_material, int n_materials,
                           const double *mu, const double *sigma, const double *sigma0,
                           ParamMatrix &P, cudaStream_t st);
// rhs[k] for S systems (omega, alfa, 1-D tables usin/ucos [S][n1d] on z1d);
// layout: interleaved ? rhs[e * S + k] : rhs[k * rhs_stride + e]
int param_rhs(const ParamMatrix &P, int S, const double *d_omega, const int *d_alfa, int n1d,
              const double *d_z1d, const double *d_usin, const double *d_ucos, double2 *d_rhs,
              long long rhs_stride, int interleaved, cudaStream_t st);
int param_to_sell(const ParamMatrix &P, double omega, SellMatrix &A, cudaStream_t st);
int param_to_block2x2(const ParamMatrix &P, double omega, Block2x2Dev &B, cudaStream_t st);
// A (complex, single system) viewed as K = Re A, M = Im A, omega = 1
int param_from_sell(const SellMatrix &A, ParamMatrix &P, cudaStream_t st);
int exclusive_scan_host(const int *d_in, int n, int *d_out, long long *total, cudaStream_t st);

}  // namespace mtgpu

// opaque handle of the device assembly (include/mtgpu.h)
struct mtgpu_assembly_s {
    mtgpu::ParamMatrix P;
    cudaStream_t st = nullptr;
    // host copies of what the folded preconditioner set-up reads
    std::vector<int> nver, nvkat, edges, bound;
    std::vector<double> xyz;
    std::vector<double> sigflag;
    std::vector<int> ig_t;
    int nver_stride = 14;
    // the SpMV variant the first survey set-up on this mesh chose, per batch
    // width (lanes): the choice depends on the mesh and the width only, so
    // later surveys on the assembly skip the autotuning
    std::map<int, int> tuned;
};
