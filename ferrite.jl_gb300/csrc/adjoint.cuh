// adjoint.cuh -- vector-Jacobian products of the assembly (heat, linear elasticity).
//
// For Phi = lambda^T (K(X, s) u - f(X)), with s_e the per-cell material factor:
//   d_cell[e] = (ds_e/drho_e) dPhi/ds_e = (ds_e/drho_e) sum_q dV psi0,
//   dPhi/dX_k  = sum_e sum_q dV Sigma grad M_k,
//   Sigma = (psi - fl) I - grad(u)^T sigma(lambda) - grad(lambda)^T sigma(u),
// psi = sigma(u) : grad(lambda) (psi0 with the unscaled material), fl = lambda(x_q) . b (heat:
// source * lambda(x_q)), grad M_k = J^-T dM_k/dxi. They follow from d(dV) = dV tr(J^-1 dJ) and
// d(grad v) = -grad(v) dJ J^-1 with J = sum_k x_k (x) dM_k/dxi. Quadrature-point geometry is
// recomputed here, not stored by the forward assembly.
//
// One lane group per cell (lane = quadrature point, as in the tile kernel's geometry). Each
// point's NG*DIM coordinate contributions and its psi0 term go to shared memory; lane k sums
// node k's contributions over the points in point order and writes them to the cell's
// contribution row; a second kernel sums each node's rows in cell order in FP64. No atomics:
// bitwise reproducible.
#pragma once
#include "tile_kernel.cuh"

namespace fe {

struct AdjArgs {
    const float* xf6;        // [n_nodes][6] float hi (x, y, z) then lo
    const double* xd3;       // [n_nodes][3]
    const float* u_f;        // mixed precision: float copies of u and lambda
    const float* l_f;
    const double* u_d;
    const double* l_d;
    const float* scale_f;    // per Ferrite cell material factor (NULL = 1)
    const double* scale_d;
    const double* dscale;    // per Ferrite cell ds/drho (NULL = 1)
    double m0, m1;           // unscaled material: heat k; elastic Lame lambda, mu
    double load[3];          // elastic body force; heat: load[0] = source
    float m0_f, m1_f, load_f[3];  // the same in FP32 (no per-point conversions)
    double* d_cell;          // [n_cells], by Ferrite cell id
    void* contrib;           // Real [rows][DIM]: per (cell, geometric node)
    int64_t row0;            // first contribution row of this subdomain
    DevStatus* status;
};

template <int K, int NQ, int PHYS, typename Real>
struct AdjT {
    static constexpr int NG = ElemT<K>::NG, DIM = ElemT<K>::DIM, GS = ElemT<K>::GS;
    static constexpr int NV = NG * DIM + 1;               // reduced values per point
    static constexpr int GROUP_REALS = NQ * NV;
    static constexpr int SMEM_BYTES = (THREADS / GS) * GROUP_REALS * (int)sizeof(Real);
};

template <int K, int NQ, int PHYS, typename Real>
__global__ void __launch_bounds__(THREADS) adjoint_kernel(const AdjArgs a, const SubDev sd, const int32_t* __restrict__ conn,
                                                         const Real* __restrict__ shp) {
    using E = ElemT<K>;
    using AT = AdjT<K, NQ, PHYS, Real>;
    constexpr int NB = E::NB, NG = E::NG, DIM = E::DIM, GS = E::GS;
    constexpr int NC = PHYS == PHYS_HEAT ? 1 : DIM;
    constexpr int NV = AT::NV;
    constexpr ShapeQ SQL = shape_q(NB, NG, DIM, (int)sizeof(Real));
    static_assert(NQ <= GS && NG <= GS, "one lane per point and per node");
    extern __shared__ __align__(16) char smem_adj[];
    const int tid = threadIdx.x, lane = tid % GS, grp = tid / GS;
    const unsigned gmask = GS >= 32 ? 0xFFFFFFFFu : (((1u << GS) - 1u) << ((tid & 31) / GS * GS));
    const int gbase = (tid & 31) - lane;
    Real* buf = (Real*)smem_adj + grp * AT::GROUP_REALS;
    Real* contrib = (Real*)a.contrib;
    const int64_t stride = (int64_t)gridDim.x * (THREADS / GS);
    for (int64_t c = (int64_t)blockIdx.x * (THREADS / GS) + grp; c < sd.n_cells; c += stride) {
        const int32_t cid = sd.cellid[c];
        // node offsets from node 0 (float: hi/lo split keeps them accurate to FP32 relative)
        Real off[NG][DIM];
        if constexpr (sizeof(Real) == 4) {
            const int nk = conn[c * NG + (lane < NG ? lane : 0)];
            const float* p = a.xf6 + (int64_t)nk * 6;
            const float h[3] = {p[0], p[1], p[2]}, l[3] = {p[3], p[4], p[5]};
            float o[DIM];
            #pragma unroll
            for (int x = 0; x < DIM; ++x) {
                const float h0 = __shfl_sync(gmask, h[x], gbase), l0 = __shfl_sync(gmask, l[x], gbase);
                o[x] = (h[x] - h0) + (l[x] - l0);
            }
            #pragma unroll
            for (int k = 0; k < NG; ++k)
                #pragma unroll
                for (int x = 0; x < DIM; ++x) off[k][x] = __shfl_sync(gmask, o[x], gbase + k);
        } else {
            const double* x0 = a.xd3 + (int64_t)conn[c * NG] * 3;
            #pragma unroll
            for (int k = 0; k < NG; ++k) {
                const double* xk = a.xd3 + (int64_t)conn[c * NG + k] * 3;
                #pragma unroll
                for (int x = 0; x < DIM; ++x) off[k][x] = xk[x] - x0[x];
            }
        }
        if (lane < NQ) {
            const int q = lane;
            const Real* Q = shp + q * SQL.qs;
            Real J[DIM * DIM];
            #pragma unroll
            for (int t = 0; t < DIM * DIM; ++t) J[t] = Real(0);
            #pragma unroll
            for (int k = 1; k < NG; ++k)
                #pragma unroll
                for (int x = 0; x < DIM; ++x)
                    #pragma unroll
                    for (int b = 0; b < DIM; ++b) J[x * DIM + b] += off[k][x] * Q[SQL.dm + k * DIM + b];
            Real dt = Mat<Real, DIM>::det(J);
            Real Ji[DIM * DIM];
            if (!(dt > Real(0))) {
                record_detj(a.status, cid, (float)dt);
                dt = Real(0);
                #pragma unroll
                for (int t = 0; t < DIM * DIM; ++t) Ji[t] = Real(0);
            } else {
                Mat<Real, DIM>::inv(J, dt, Ji);
            }
            const Real dV = dt * Q[SQL.w];
            // gradients of u and lambda (G[comp][d] = d v_comp / d x_d) and lambda at the point
            Real Gu[NC * DIM], Gl[NC * DIM], lq[NC];
            #pragma unroll
            for (int t = 0; t < NC * DIM; ++t) { Gu[t] = Real(0); Gl[t] = Real(0); }
            #pragma unroll
            for (int t = 0; t < NC; ++t) lq[t] = Real(0);
            for (int i = 0; i < NB; ++i) {
                Real g[DIM];
                #pragma unroll
                for (int b = 0; b < DIM; ++b) {
                    g[b] = Real(0);
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x) g[b] += Q[SQL.dn + i * DIM + x] * Ji[x * DIM + b];
                }
                const Real Ni = Q[SQL.n + i];
                const int64_t base = (int64_t)sd.ents[c * NB + i] * NC;
                #pragma unroll
                for (int m = 0; m < NC; ++m) {
                    Real ui, li;
                    if constexpr (sizeof(Real) == 4) { ui = a.u_f[base + m]; li = a.l_f[base + m]; }
                    else { ui = a.u_d[base + m]; li = a.l_d[base + m]; }
                    lq[m] += Ni * li;
                    #pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        Gu[m * DIM + d] += ui * g[d];
                        Gl[m * DIM + d] += li * g[d];
                    }
                }
            }
            // flux / stress with the unscaled material
            Real Su[NC * DIM], Sl[NC * DIM];
            if constexpr (PHYS == PHYS_HEAT) {
                #pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    Su[d] = pconst<Real>(a.m0, a.m0_f) * Gu[d];
                    Sl[d] = pconst<Real>(a.m0, a.m0_f) * Gl[d];
                }
            } else {
                Real tu = 0, tl = 0;
                #pragma unroll
                for (int d = 0; d < DIM; ++d) { tu += Gu[d * DIM + d]; tl += Gl[d * DIM + d]; }
                const Real lam = pconst<Real>(a.m0, a.m0_f), mu = pconst<Real>(a.m1, a.m1_f);
                #pragma unroll
                for (int x = 0; x < DIM; ++x)
                    #pragma unroll
                    for (int y = 0; y < DIM; ++y) {
                        Su[x * DIM + y] = mu * (Gu[x * DIM + y] + Gu[y * DIM + x]) + (x == y ? lam * tu : Real(0));
                        Sl[x * DIM + y] = mu * (Gl[x * DIM + y] + Gl[y * DIM + x]) + (x == y ? lam * tl : Real(0));
                    }
            }
            Real psi0 = 0;
            #pragma unroll
            for (int t = 0; t < NC * DIM; ++t) psi0 += Su[t] * Gl[t];
            Real s = Real(1);
            if (a.scale_d) {
                if constexpr (sizeof(Real) == 4) s = a.scale_f[cid];
                else s = a.scale_d[cid];
            }
            Real fl = 0;
            #pragma unroll
            for (int m = 0; m < NC; ++m) fl += lq[m] * pconst<Real>(a.load[m], a.load_f[m]);
            Real Sg[DIM * DIM];
            #pragma unroll
            for (int b = 0; b < DIM; ++b)
                #pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    Real v = Real(0);
                    #pragma unroll
                    for (int m = 0; m < NC; ++m) v += Gu[m * DIM + b] * Sl[m * DIM + d] + Gl[m * DIM + b] * Su[m * DIM + d];
                    Sg[b * DIM + d] = (b == d ? s * psi0 - fl : Real(0)) - s * v;
                }
            Real* out = buf + q * NV;
            #pragma unroll
            for (int k = 0; k < NG; ++k) {
                Real gM[DIM];
                #pragma unroll
                for (int b = 0; b < DIM; ++b) {
                    gM[b] = Real(0);
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x) gM[b] += Q[SQL.dm + k * DIM + x] * Ji[x * DIM + b];
                }
                #pragma unroll
                for (int b = 0; b < DIM; ++b) {
                    Real v = Real(0);
                    #pragma unroll
                    for (int d = 0; d < DIM; ++d) v += Sg[b * DIM + d] * gM[d];
                    out[k * DIM + b] = dV * v;
                }
            }
            out[NV - 1] = dV * psi0;
        }
        __syncwarp(gmask);
        if (lane < NG) {
            Real v[DIM];
            #pragma unroll
            for (int b = 0; b < DIM; ++b) v[b] = Real(0);
            for (int q = 0; q < NQ; ++q)
                #pragma unroll
                for (int b = 0; b < DIM; ++b) v[b] += buf[q * NV + lane * DIM + b];
            Real* dst = contrib + (a.row0 + c * NG + lane) * DIM;
            #pragma unroll
            for (int b = 0; b < DIM; ++b) dst[b] = v[b];
        }
        if (lane == 0) {
            Real g = Real(0);
            for (int q = 0; q < NQ; ++q) g += buf[q * NV + NV - 1];
            a.d_cell[cid] = (a.dscale ? a.dscale[cid] : 1.0) * (double)g;
        }
        __syncwarp(gmask);  // the next cell overwrites the buffer
    }
}

// dX[n][b] = sum over the node's (cell, node) rows, in cell order, in FP64
template <typename Real>
__global__ void adjoint_node_sum(const int64_t* __restrict__ ptr, const int32_t* __restrict__ rows, const Real* __restrict__ contrib,
                                 int dim, int64_t n_nodes, double* __restrict__ dX) {
    const int64_t n_out = n_nodes * dim;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n_out; idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = idx / dim, b = idx - n * dim;
        double s = 0.0;
        for (int64_t e = ptr[n]; e < ptr[n + 1]; ++e) s += (double)contrib[(int64_t)rows[e] * dim + b];
        dX[idx] = s;
    }
}

}  // namespace fe
