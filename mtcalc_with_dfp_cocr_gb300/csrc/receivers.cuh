// Receiver handle shared by the receiver (receivers.cu) and adjoint
// (adjoint.cu) kernels.
#pragma once
#include "assemble.cuh"

namespace mtgpu {

// grow-only device buffer
template <class T>
int ensure(T **p, size_t *cap, size_t n)
{
    if (n <= *cap && *p) return MTGPU_OK;
    dev_free(*p);
    *cap = 0;
    int rc = dev_alloc(p, n);
    if (rc) return rc;
    *cap = n;
    return MTGPU_OK;
}

// elem[r] = the lowest brick whose box [vertex 0, vertex 7] grown by `grow`
// holds receiver r (INT_MAX: none); skip_air leaves out material 0
int locate_receivers(const ParamMatrix &P, int nrec, const double *d_rec, double grow,
                     bool skip_air, int *d_elem, cudaStream_t st);

// Subdomain smoothing of the receiver output (smoothing.cu)
struct Smoothing {
    int levels = 5;
    int nsub = 0;                    // [0]: curl A over all materials; [1..]: A per material
    int npad = 0, ncell = 0, nblk = 0;
    std::vector<int> sub_cells, sub_nodes, sub_material;
    int *d_cell = nullptr, *d_cell_sub = nullptr;     // [ncell] global brick, subdomain
    double *d_cell_g = nullptr;                       // [ncell] row sum of the brick mass matrix
    int *d_nc_ptr = nullptr, *d_nc = nullptr;         // padded node -> bricks (d_cell index)
    int *d_mptr = nullptr, *d_mcol = nullptr;         // nodal mass matrix, padded rows
    double *d_mval = nullptr, *d_mdiag = nullptr;
    int *d_blk_sub = nullptr;                         // [nblk] subdomain of each node block
    int *d_rn = nullptr;                              // [nrec][2][8] nodes (curl A, A); -1 none
    double *d_rw = nullptr;                           // [nrec][2][8] trilinear weights
    int S_cap = 0;
    double *d_val = nullptr, *d_x = nullptr, *d_r = nullptr, *d_z = nullptr, *d_p = nullptr,
           *d_q = nullptr, *d_scal = nullptr;
    int *d_done = nullptr, *d_active = nullptr;
    int iterations = 0;
    void release();
};

int smoothing_build(Smoothing &sm, const ::mtgpu_assembly_s &a, int nrec,
                    const double *xyz_rec, cudaStream_t st);
// smoothed A and curl A -> total fields, as mtgpu_receivers_fields (d_loc:
// the receivers' local coordinates, .w the depth)
int smoothing_fields(Smoothing &sm, const ParamMatrix &P, int nrec, int S, long long x_stride,
                     const double2 *d_x, const double *d_omega, const int *d_alfa, int n1d,
                     const double *d_z1d, const double *d_us, const double *d_uc,
                     const double4 *d_loc, double2 *d_e, double2 *d_h, double2 *d_scal,
                     cudaStream_t st);

}  // namespace mtgpu

struct mtgpu_receivers_s {
    cudaStream_t st = nullptr;
    int nrec = 0, nb = 0, n_unlocated = 0;
    int *d_elem = nullptr;          // containing brick, -1 none
    int *d_edge = nullptr;          // [nrec][12] the brick's edges
    double4 *d_loc = nullptr;       // local coordinates xi, eta, zeta; receiver z
    double4 *d_h = nullptr;         // brick sizes
    std::vector<int> elem;          // host copy of d_elem
    std::vector<double> rec;        // receivers [nrec][3]
    const mtgpu_assembly_s *asm_ = nullptr;   // the assembly they were located in
    int output = 0;                 // MTGPU_OUTPUT_DIRECT / MTGPU_OUTPUT_SMOOTH
    mtgpu::Smoothing *sm = nullptr;
    // per-call inputs (grow-only)
    double *d_omega = nullptr, *d_tab = nullptr;
    int *d_int = nullptr;
    size_t cap_omega = 0, cap_tab = 0, cap_int = 0;
    // adjoint: per-(system, receiver, local edge) contributions and the
    // edges they land on, grouped by edge in ascending (receiver, slot) order
    double2 *d_contrib = nullptr;
    double *d_misfit = nullptr;
    size_t cap_contrib = 0, cap_misfit = 0;
    int n_touch = 0;
    int *d_touch_ptr = nullptr, *d_touch_edge = nullptr, *d_touch_slot = nullptr;
};
