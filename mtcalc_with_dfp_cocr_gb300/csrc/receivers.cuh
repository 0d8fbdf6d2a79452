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

}  // namespace mtgpu

struct mtgpu_receivers_s {
    cudaStream_t st = nullptr;
    int nrec = 0, nb = 0, n_unlocated = 0;
    int *d_elem = nullptr;          // containing brick, -1 none
    int *d_edge = nullptr;          // [nrec][12] the brick's edges
    double4 *d_loc = nullptr;       // local coordinates xi, eta, zeta; receiver z
    double4 *d_h = nullptr;         // brick sizes
    std::vector<int> elem;          // host copy of d_elem
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
