// The folded preconditioner of the iteration in one kernel on tensor meshes,
// included by survey.cu after k_node / k_edge.
//
// k_node (h = D_S G (z + beta a)) and k_edge (p = s + beta p, a = z + beta a,
// w = D_A a + G^T h, (a, w)) are two passes over the vectors with h in
// global memory between them.  On a tensor mesh numbered as
// RegularMeshBuilder numbers it, with every interior node a row of G (in
// node order) and the Dirichlet edges on the outer surface, a node's G row
// is its six edges and an edge's G^T row its two nodes, so one kernel does
// both: a block owns a tile of TX x TY node columns and marches along z;
// per plane it stages a_new = z + beta a of the edges owned by the plane's
// nodes (tile plus a one-node halo), computes h of the plane's nodes (tile
// plus one on the + side) into shared memory, and produces p, a, w of the
// edges owned by the previous plane's nodes.  Every vector crosses HBM once;
// h never leaves the SM.
//
// a is read (a_in) and written (a_out) in different buffers: the halo of a
// tile reads a neighbour tile's edges.  The sums run in the order of k_node
// (a node's edges by increasing number: -z, -y, -x, +x, +y, +z) and k_edge
// (D_A a, then the first node's -1/2 h, then the second's +1/2 h), so p, a
// and w equal the two-kernel form's to the last bit; the grid sum (a, w)
// groups its terms by tile and so rounds differently.

template <int SP>
struct PrecTile {
    static constexpr int SB = SP >= 2 ? 2 : 1;
    static constexpr int TX = 32;
    static constexpr int TY = SB == 1 ? 8 : 4;
    static constexpr int NT = TX * TY * SB;
    static constexpr int NX = TX + 2, NY = TY + 2, NS = NX * NY;
    // float4 slots: a_new of x/y edges [2 planes][2][SB][NS], of z edges
    // [2 layers][SB][NS], h [2 planes][SB][NS]
    static constexpr int OFF_AXY = 0;
    static constexpr int OFF_AZ = OFF_AXY + 2 * 2 * SB * NS;
    static constexpr int OFF_H = OFF_AZ + 2 * SB * NS;
    static constexpr int SLOTS = OFF_H + 2 * SB * NS;
    static constexpr int SMEM = SLOTS * 16;
    static_assert(NT * 2 * 8 <= SMEM, "staging fits");
};

struct PrecGrid {
    int tiles_x, tiles_y, zchunks, groups, kz;
};

template <int SP>
__global__ void __launch_bounds__(PrecTile<SP>::NT)
k_prec_tile(MF M, PrecGrid G, const float4 *__restrict__ ds, const float4 *__restrict__ da,
            const float4 *__restrict__ s, const float4 *__restrict__ z,
            const float4 *__restrict__ a_in, float4 *__restrict__ a_out, float4 *__restrict__ p,
            float4 *__restrict__ w, float4 *__restrict__ x, SysState *sys, double *partials)
{
    pdl_wait();
    using C = PrecTile<SP>;
    constexpr int SB = C::SB, TX = C::TX, TY = C::TY, NT = C::NT, NX = C::NX, NS = C::NS;
    extern __shared__ __align__(16) float4 sh[];
    float4 *const AXY = sh + C::OFF_AXY, *const AZ = sh + C::OFF_AZ, *const H = sh + C::OFF_H;
    auto at2 = [](int p) { return (p + 2) & 1; };
    auto axy = [&](int pl, int d, int ii, int jj, int u) -> float4 & {
        return AXY[((at2(pl) * 2 + d) * SB + u) * NS + jj * NX + ii];
    };
    auto az = [&](int ly, int ii, int jj, int u) -> float4 & {
        return AZ[(at2(ly) * SB + u) * NS + jj * NX + ii];
    };
    auto hh = [&](int pl, int ii, int jj, int u) -> float4 & {
        return H[(at2(pl) * SB + u) * NS + jj * NX + ii];
    };

    int b = blockIdx.x;
    const int grp = b % G.groups;
    b /= G.groups;
    const int tx = b % G.tiles_x;
    b /= G.tiles_x;
    const int ty = b % G.tiles_y;
    const int zc = b / G.tiles_y;
    const int i0 = tx * TX, j0 = ty * TY, sys0 = grp * SB;
    const int nx = M.nx, ny = M.ny, nz = M.nz;
    const int k0 = zc * G.kz, k1 = min(k0 + G.kz, nz);
    const int tid = threadIdx.x;
    const int u_me = tid / (TX * TY), ti = tid % TX, tj = (tid / TX) % TY;
    // beta of the block's systems (two at most), selected without indexing
    const dfc be0 = from_d2(sys[sys0].beta);
    const dfc be1 = SB > 1 ? from_d2(sys[sys0 + SB - 1].beta) : be0;
    auto beta_of = [&](int u) { return u ? be1 : be0; };

    // a_new of the edges owned by the nodes of plane P (x, y on P; z of
    // layer P) over the halo frame; absent edges 0
    auto load_plane = [&](int P) {
        for (int q = tid; q < NS * 3 * SB; q += NT) {
            const int u = q % SB, d = (q / SB) % 3, slot = q / (3 * SB);
            const int ii = slot % NX, jj = slot / NX;
            const int i = i0 - 1 + ii, j = j0 - 1 + jj;
            dfc v{df{0.f, 0.f}, df{0.f, 0.f}};
            if (P >= 0 && P < nz && i >= 0 && i < nx && j >= 0 && j < ny) {
                const int ex = i < nx - 1, ey = j < ny - 1, ezp = P < nz - 1;
                if (d == 0 ? ex : (d == 1 ? ey : ezp)) {
                    int e = mf_line(M, j, P) + i * (1 + ey + ezp);
                    if (d >= 1) e += ex;
                    if (d == 2) e += ey;
                    const long long idx = (long long)e * SP + sys0 + u;
                    v = caxpy(from4(__ldg(z + idx)), beta_of(u), from4(__ldg(a_in + idx)));
                }
            }
            if (d < 2) axy(P, d, ii, jj, u) = to4(v);
            else az(P, ii, jj, u) = to4(v);
        }
    };
    // h of the nodes of plane P on the frame nodes ii in [1, TX+1], jj in [1, TY+1]
    auto node_h = [&](int P) {
        constexpr int n = (TX + 1) * (TY + 1);
        for (int q = tid; q < n * SB; q += NT) {
            const int u = q / n, c = q % n, ii = 1 + c % (TX + 1), jj = 1 + c / (TX + 1);
            const int i = i0 - 1 + ii, j = j0 - 1 + jj;
            float4 out = f4zero();
            if (i >= 1 && i < nx - 1 && j >= 1 && j < ny - 1 && P >= 1 && P < nz - 1) {
                const long long row = ((long long)(P - 1) * (ny - 2) + (j - 1)) * (nx - 2) + (i - 1);
                const dfc t[6] = {from4(az(P - 1, ii, jj, u)), from4(axy(P, 1, ii, jj - 1, u)),
                                  from4(axy(P, 0, ii - 1, jj, u)), from4(axy(P, 0, ii, jj, u)),
                                  from4(axy(P, 1, ii, jj, u)), from4(az(P, ii, jj, u))};
                acc hr, hi;
#pragma unroll
                for (int m = 0; m < 6; m++) {
                    const float g = m < 3 ? 0.5f : -0.5f;
                    hr.macf(t[m].re, g);
                    hi.macf(t[m].im, g);
                }
                out = to4(cmul(dfc{hr.get(), hi.get()}, from4(__ldg(ds + row * SP + sys0 + u))));
            }
            hh(P, ii, jj, u) = out;
        }
    };

    load_plane(k0 - 1);
    load_plane(k0);
    __syncthreads();
    node_h(k0);
    __syncthreads();

    const int ii = ti + 1, jj = tj + 1;
    const int i = i0 + ti, j = j0 + tj;
    const int kme = sys0 + u_me;
    const dfc bme = beta_of(u_me);
    // the previous iteration's x += alpha p, as in k_edge
    const bool xpme = sys[kme].xp;
    const dfc alme = from_d2(sys[kme].alpha);
    const bool col = i < nx && j < ny && sys[kme].status == kRun;
    acc awr, awi;
    for (int k = k0; k < k1; k++) {
        load_plane(k + 1);
        __syncthreads();
        node_h(k + 1);
        __syncthreads();
        if (col) {
            const int ex = i < nx - 1, ey = j < ny - 1, ezp = k < nz - 1;
            const int base = mf_line(M, j, k) + i * (1 + ey + ezp);
#pragma unroll
            for (int d = 0; d < 3; d++) {
                if (!(d == 0 ? ex : (d == 1 ? ey : ezp))) continue;
                const long long idx = (long long)(base + (d == 0 ? 0 : (d == 1 ? ex : ex + ey))) * SP + kme;
                const float4 srcv = __ldg(s + idx), dav = __ldg(da + idx), pv = p[idx];
                const dfc an = from4(d == 0 ? axy(k, 0, ii, jj, u_me)
                                            : (d == 1 ? axy(k, 1, ii, jj, u_me) : az(k, ii, jj, u_me)));
                // the edge's nodes: (i, j, k) first, its +d neighbour second;
                // G rows exist for interior nodes only (h is 0 elsewhere)
                const bool in0 = i >= 1 && i < nx - 1 && j >= 1 && j < ny - 1 && k >= 1 && k < nz - 1;
                const int i1 = i + (d == 0), j1 = j + (d == 1), k1n = k + (d == 2);
                const bool in1 = i1 >= 1 && i1 < nx - 1 && j1 >= 1 && j1 < ny - 1 && k1n >= 1 &&
                                 k1n < nz - 1;
                const float4 h0 = hh(k, ii, jj, u_me);
                const float4 h1 = d == 2 ? hh(k + 1, ii, jj, u_me)
                                         : hh(k, ii + (d == 0), jj + (d == 1), u_me);
                if (xpme) x[idx] = to4(caxpy(from4(x[idx]), alme, from4(pv)));
                p[idx] = to4(caxpy(from4(srcv), bme, from4(pv)));
                a_out[idx] = to4(an);
                const dfc dv = cmul(an, from4(dav));
                acc wr, wi;
                wr.h = dv.re.h; wr.l = dv.re.l;
                wi.h = dv.im.h; wi.l = dv.im.l;
                if (in0) {
                    wr.macf(df{h0.x, h0.y}, -0.5f);
                    wi.macf(df{h0.z, h0.w}, -0.5f);
                }
                if (in1) {
                    wr.macf(df{h1.x, h1.y}, 0.5f);
                    wi.macf(df{h1.z, h1.w}, 0.5f);
                }
                const dfc wn{wr.get(), wi.get()};
                w[idx] = to4(wn);
                awr.mac(an.re, wn.re);
                awr.mac(neg(an.im), wn.im);
                awi.mac(an.re, wn.im);
                awi.mac(an.im, wn.re);
            }
        }
        __syncthreads();   // the next plane's staging overwrites the rings read above
    }
    // per-system (a, w) in a fixed order, then the grid sum and alpha as k_edge
    double *const red = reinterpret_cast<double *>(sh);
    red[tid] = awr.to_double();
    red[NT + tid] = awi.to_double();
    __syncthreads();
    double v[2] = {0.0, 0.0};
    if (tid < SP) {
        const int u = tid - sys0;
        if (u >= 0 && u < SB)
            for (int t = u * TX * TY; t < (u + 1) * TX * TY; t++) {
                v[0] += red[t];
                v[1] += red[NT + t];
            }
    }
    __shared__ double tot[2][32];
    if (sys_grid_sum<SP, 2, NT>(v, partials, &sys[0].ticket[1], tot) && threadIdx.x < SP) {
        SysState &q = sys[threadIdx.x];
        if (q.status == kRun) {
            const double2 aw = make_double2(tot[0][threadIdx.x], tot[1][threadIdx.x]);
            if (fabs(aw.x) < 1e-40 && fabs(aw.y) < 1e-40) q.status = MTGPU_DIV_BY_ZERO;
            else q.alpha = cdiv(q.zs, aw);
        }
    }
}
