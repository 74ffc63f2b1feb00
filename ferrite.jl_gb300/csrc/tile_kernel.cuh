// tile_kernel.cuh -- the owner-tile assembly kernel.
//
// One CTA assembles one tile: the nzval ranges of a compact set of dof entities.
//   0. entity table + zeroed accumulators in shared memory; reference shape tables staged
//      into shared memory with a TMA bulk copy (cp.async.bulk + mbarrier).
//   1. for every wave (cells that share no owned entity) and chunk of its cells:
//      A. one thread per (cell, quadrature point): Jacobian from the node coordinates
//         (split float hi+lo, so cell-size differences keep FP32 relative accuracy), detJ,
//         J^-1, and the physical gradients scaled by sqrt(detJ*w) -> shared-memory table.
//         Cells whose Jacobian condition number exceeds a threshold are redone in FP64.
//      B. one lane group per (cell, owned base function j), lane i = row base function:
//         the nc x nc block of Ke (rows of i, columns of j) and, on lane i == j, fe_j;
//         added into the accumulator entries of the owning columns (compensated FP32 pair
//         = FP64-class accumulation). Lanes of a group hit distinct rows; groups of a wave
//         hit distinct columns, so there are no conflicting updates and the summation order
//         of every entry is fixed by the plan.
//   2. write-out: each owned nzval / f entry stored once, coalesced, streaming.
//
// Reference correspondence: step A is reinit!(cv, x) (src/FEValues/CellValues.jl:122-140,
// GeometryMapping.jl:124-130, FunctionValues.jl:186-192); step B is the element routine
// (heat_equation.jl:143-164, threaded_assembly.jl:105-119, hyperelasticity.jl:241-276)
// fused with assemble! (src/assembler.jl:322-457); step 2 replaces fillzero! + the
// scattered addindex! updates (src/arrayutils.jl:100-152).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.h"
#include "dfloat.h"

namespace fe {

// ---------------------------------------------------------------------------------------
// element traits
// ---------------------------------------------------------------------------------------
template <int K> struct ElemT;
template <> struct ElemT<KIND_TRI3>   { static constexpr int DIM = 2, NG = 3, NB = 3, GS = 4; };
template <> struct ElemT<KIND_QUAD4>  { static constexpr int DIM = 2, NG = 4, NB = 4, GS = 4; };
template <> struct ElemT<KIND_TET4>   { static constexpr int DIM = 3, NG = 4, NB = 4, GS = 4; };
template <> struct ElemT<KIND_HEX8>   { static constexpr int DIM = 3, NG = 8, NB = 8, GS = 8; };
template <> struct ElemT<KIND_WEDGE6> { static constexpr int DIM = 3, NG = 6, NB = 6, GS = 8; };
template <> struct ElemT<KIND_HEX27>  { static constexpr int DIM = 3, NG = 8, NB = 27, GS = 32; };
template <> struct ElemT<KIND_QUAD9>  { static constexpr int DIM = 2, NG = 4, NB = 9, GS = 16; };

constexpr int PHYS_HEAT = 1, PHYS_ELASTIC = 2, PHYS_NEO = 3;
constexpr int NEO_EXTRA = 32;  // per (cell, qp): T = S + c1 C^-1 (9), B = F^-T (9), c1, 2c2, P (9), pad
constexpr int THREADS = 256;

struct __align__(16) D4 {
    double x, y, z, w;
};
template <typename Real> struct Vec4T;
template <> struct Vec4T<float> { using type = float4; };
template <> struct Vec4T<double> { using type = D4; };
template <typename Real> struct AccT;
template <> struct AccT<float> { using type = float2; };   // (hi, lo) compensated pair
template <> struct AccT<double> { using type = double; };

// ---------------------------------------------------------------------------------------
// accumulation
// ---------------------------------------------------------------------------------------
// TwoSum (Knuth): s + e == a + x exactly; the rounding errors collect in the low word.
__device__ __forceinline__ void acc_add(float2& a, float x) {
    const float s = __fadd_rn(a.x, x);
    const float bb = __fsub_rn(s, a.x);
    const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    a.x = s;
    a.y = __fadd_rn(a.y, e);
}
__device__ __forceinline__ void acc_add(double& a, double x) { a += x; }

__device__ __forceinline__ double acc_value(float2 a) { return pair_to_double(a.x, a.y); }
__device__ __forceinline__ double acc_value(double a) { return a; }
__device__ __forceinline__ void acc_zero(float2& a) { a = make_float2(0.f, 0.f); }
__device__ __forceinline__ void acc_zero(double& a) { a = 0.0; }
__device__ __forceinline__ void acc_set(float2& a, double v) {
    const float h = (float)v;
    a = make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ void acc_set(double& a, double v) { a = v; }

// ---------------------------------------------------------------------------------------
// small dense helpers
// ---------------------------------------------------------------------------------------
template <typename R, int D> struct Mat;
template <typename R> struct Mat<R, 3> {
    static __device__ __forceinline__ R det(const R* J) {
        return J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) + J[2] * (J[3] * J[7] - J[4] * J[6]);
    }
    static __device__ __forceinline__ void inv(const R* J, R dt, R* Ji) {
        const R id = R(1) / dt;
        Ji[0] = (J[4] * J[8] - J[5] * J[7]) * id;
        Ji[1] = -(J[1] * J[8] - J[2] * J[7]) * id;
        Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
        Ji[3] = -(J[3] * J[8] - J[5] * J[6]) * id;
        Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id;
        Ji[5] = -(J[0] * J[5] - J[2] * J[3]) * id;
        Ji[6] = (J[3] * J[7] - J[4] * J[6]) * id;
        Ji[7] = -(J[0] * J[7] - J[1] * J[6]) * id;
        Ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
    }
};
template <typename R> struct Mat<R, 2> {
    static __device__ __forceinline__ R det(const R* J) { return J[0] * J[3] - J[1] * J[2]; }
    static __device__ __forceinline__ void inv(const R* J, R dt, R* Ji) {
        const R id = R(1) / dt;
        Ji[0] = J[3] * id; Ji[1] = -J[1] * id;
        Ji[2] = -J[2] * id; Ji[3] = J[0] * id;
    }
};

__device__ __forceinline__ void record_detj(DevStatus* st, int32_t cellid, float detJ) {
    const unsigned long long key = ((unsigned long long)(uint32_t)cellid << 32) | __float_as_uint(detJ);
    atomicMin(&st->detj_key, key);
}
__device__ __forceinline__ void record_miss(DevStatus* st, int32_t cellid, int I, int J) {
    const unsigned long long key = ((unsigned long long)(uint32_t)cellid << 32) | ((unsigned)I << 16) | (unsigned)J;
    atomicMin(&st->miss_key, key);
}

// Neo-Hooke at one point in FP32 without cancellation for small strains:
// X = C - I = H + H^T + H^T H, det C - 1 from the invariants of X, I - C^-1 = C^-1 X.
// Outputs T = S + c1 C^-1, B = F^-T, c1, 2 c2 and P = F S such that
// dP/dF_aJbL = delta_ab T_JL + c1 B_aL B_bJ + 2c2 B_aJ B_bL (hyperelasticity.jl:157-176, 254).
template <typename R>
__device__ __forceinline__ void neo_hooke_point(R mu, R lam, const R* H, R* out) {
    R F[9], X[9], C[9], Ci[9];
    #pragma unroll
    for (int a = 0; a < 9; ++a) F[a] = H[a];
    F[0] += R(1); F[4] += R(1); F[8] += R(1);
    #pragma unroll
    for (int I = 0; I < 3; ++I)
        #pragma unroll
        for (int J = 0; J < 3; ++J) {
            R hh = 0;
            #pragma unroll
            for (int k = 0; k < 3; ++k) hh += H[k * 3 + I] * H[k * 3 + J];
            X[I * 3 + J] = H[I * 3 + J] + H[J * 3 + I] + hh;
            C[I * 3 + J] = X[I * 3 + J] + (I == J ? R(1) : R(0));
        }
    const R trX = X[0] + X[4] + X[8];
    R trX2 = 0;
    #pragma unroll
    for (int I = 0; I < 3; ++I)
        #pragma unroll
        for (int J = 0; J < 3; ++J) trX2 += X[I * 3 + J] * X[J * 3 + I];
    const R detCm1 = trX + R(0.5) * (trX * trX - trX2) + Mat<R, 3>::det(X);
    const R detC = R(1) + detCm1;
    Mat<R, 3>::inv(C, detC, Ci);
    const R Jd = sqrt(detC);
    const R Jm1 = detCm1 / (Jd + R(1));
    R S[9];
    #pragma unroll
    for (int I = 0; I < 3; ++I)
        #pragma unroll
        for (int J = 0; J < 3; ++J) {
            R cx = 0;
            #pragma unroll
            for (int k = 0; k < 3; ++k) cx += Ci[I * 3 + k] * X[k * 3 + J];
            S[I * 3 + J] = mu * cx + lam * Jm1 * Jd * Ci[I * 3 + J];
        }
    const R c1 = mu - lam * Jm1 * Jd;
    const R c2x2 = lam * (R(2) * Jd - R(1)) * Jd;
    // B = F^-T = F C^-1
    #pragma unroll
    for (int a = 0; a < 3; ++a)
        #pragma unroll
        for (int L = 0; L < 3; ++L) {
            R b = 0;
            #pragma unroll
            for (int I = 0; I < 3; ++I) b += F[a * 3 + I] * Ci[I * 3 + L];
            out[9 + a * 3 + L] = b;
        }
    #pragma unroll
    for (int a = 0; a < 9; ++a) out[a] = S[a] + c1 * Ci[a];
    out[18] = c1;
    out[19] = c2x2;
    #pragma unroll
    for (int a = 0; a < 3; ++a)
        #pragma unroll
        for (int J = 0; J < 3; ++J) {
            R p = 0;
            #pragma unroll
            for (int I = 0; I < 3; ++I) p += F[a * 3 + I] * S[I * 3 + J];
            out[20 + a * 3 + J] = p;
        }
}

// ---------------------------------------------------------------------------------------
// per-CTA shared memory views
// ---------------------------------------------------------------------------------------
template <typename Real>
struct Smem {
    using Acc = typename AccT<Real>::type;
    using V4 = typename Vec4T<Real>::type;
    Acc* acc;     // [acc_cap]
    Acc* facc;    // [ent_cap * nc]
    int4* etab;   // [ent_cap]: (acc_col, collen, f_off, -)
    Real* shape;  // staged reference tables of all subdomains
    char* chunk;  // per-chunk cell tables
};

// bytes of one cell's chunk table
template <int K, int NQ, int PHYS, typename Real>
__host__ __device__ constexpr int cell_table_bytes() {
    return (NQ * ElemT<K>::NB * (int)sizeof(typename Vec4T<Real>::type) + NQ * (int)sizeof(Real) + 4 * (int)sizeof(Real) +
            (PHYS == PHYS_NEO ? NQ * NEO_EXTRA * (int)sizeof(Real) : 0) + 15) & ~15;
}

// shape table block per subdomain: w[NQ], N[NQ][NB], dN[NQ][NB][DIM], dM[NQ][NG][DIM],
// each padded to a multiple of 2 doubles (16 bytes)
__host__ __device__ inline int pad16(int bytes) { return (bytes + 15) & ~15; }
template <typename Real>
__host__ __device__ inline int shape_block_bytes(int nq, int nb, int ng, int dim) {
    return pad16(nq * (int)sizeof(Real)) + pad16(nq * nb * (int)sizeof(Real)) + pad16(nq * nb * dim * (int)sizeof(Real)) +
           pad16(nq * ng * dim * (int)sizeof(Real));
}

// ---------------------------------------------------------------------------------------
// one wave of one element kind
// ---------------------------------------------------------------------------------------
template <int K, int NQ, int PHYS, typename Real>
__device__ __forceinline__ void process_wave(const KernelArgs& a, const SubDev& sd, const Real* shp, const WaveDesc& w,
                                             const Smem<Real>& sm) {
    using E = ElemT<K>;
    using V4 = typename Vec4T<Real>::type;
    constexpr int NB = E::NB, NG = E::NG, DIM = E::DIM, GS = E::GS;
    constexpr int NC_MAX = DIM;
    const int nc = a.nc;
    const Real* w_s = shp;
    const Real* N_s = (const Real*)((const char*)w_s + pad16(NQ * sizeof(Real)));
    const Real* dN_s = (const Real*)((const char*)N_s + pad16(NQ * NB * sizeof(Real)));
    const Real* dM_s = (const Real*)((const char*)dN_s + pad16(NQ * NB * DIM * sizeof(Real)));
    constexpr int TB = cell_table_bytes<K, NQ, PHYS, Real>();
    const int chunk = a.chunk_cells;
    const int tid = threadIdx.x;
    for (int s0 = 0; s0 < w.n_cells; s0 += chunk) {
        const int nchunk = min(chunk, w.n_cells - s0);
        // ---------------- phase A: geometry of the chunk's cells ----------------
        for (int idx = tid; idx < nchunk * NQ; idx += THREADS) {
            const int slot = idx / NQ, q = idx - slot * NQ;
            const int cell = a.wave_cells[w.cell_begin + s0 + slot];
            char* tb = sm.chunk + slot * TB;
            V4* grad = (V4*)tb;                                   // [NQ][NB]
            Real* sq = (Real*)(tb + NQ * NB * sizeof(V4));        // [NQ]
            Real* cellp = sq + NQ;                                // [4]
            Real* neo = cellp + 4;                                // [NQ][NEO_EXTRA]
            const int32_t* cn = sd.conn + (int64_t)cell * NG;
            Real J[DIM * DIM];
            #pragma unroll
            for (int t = 0; t < DIM * DIM; ++t) J[t] = Real(0);
            int n0 = cn[0];
            if constexpr (sizeof(Real) == 4) {
                float h0[DIM], l0[DIM];
                #pragma unroll
                for (int x = 0; x < DIM; ++x) { h0[x] = __ldg(a.xh[x] + n0); l0[x] = __ldg(a.xl[x] + n0); }
                #pragma unroll
                for (int k = 1; k < NG; ++k) {
                    const int nk = cn[k];
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x) {
                        const float off = (__ldg(a.xh[x] + nk) - h0[x]) + (__ldg(a.xl[x] + nk) - l0[x]);
                        #pragma unroll
                        for (int b = 0; b < DIM; ++b) J[x * DIM + b] += off * dM_s[(q * NG + k) * DIM + b];
                    }
                }
            } else {
                double x0[DIM];
                #pragma unroll
                for (int x = 0; x < DIM; ++x) x0[x] = a.xd[(int64_t)n0 * a.dim + x];
                #pragma unroll
                for (int k = 1; k < NG; ++k) {
                    const int nk = cn[k];
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x) {
                        const double off = a.xd[(int64_t)nk * a.dim + x] - x0[x];
                        #pragma unroll
                        for (int b = 0; b < DIM; ++b) J[x * DIM + b] += off * dM_s[(q * NG + k) * DIM + b];
                    }
                }
            }
            Real dt = Mat<Real, DIM>::det(J);
            Real Ji[DIM * DIM];
            bool bad = !(dt > Real(0));
            if (!bad) Mat<Real, DIM>::inv(J, dt, Ji);
            if constexpr (sizeof(Real) == 4) {
                // FP64 Jacobian for flagged cells: Frobenius condition estimate
                float nJ = 0, nJi = 0;
                if (!bad) {
                    #pragma unroll
                    for (int t = 0; t < DIM * DIM; ++t) { nJ += J[t] * J[t]; nJi += Ji[t] * Ji[t]; }
                }
                if (bad || sqrtf(nJ * nJi) > a.phys.cond_threshold * DIM) {
                    double Jd[DIM * DIM], Jid[DIM * DIM];
                    #pragma unroll
                    for (int t = 0; t < DIM * DIM; ++t) Jd[t] = 0.0;
                    double x0[DIM];
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x) x0[x] = a.xd[(int64_t)n0 * a.dim + x];
                    for (int k = 1; k < NG; ++k) {
                        const int nk = cn[k];
                        for (int x = 0; x < DIM; ++x) {
                            const double off = a.xd[(int64_t)nk * a.dim + x] - x0[x];
                            for (int b = 0; b < DIM; ++b) Jd[x * DIM + b] += off * sd.dM_d[(q * NG + k) * DIM + b];
                        }
                    }
                    const double dtd = Mat<double, DIM>::det(Jd);
                    bad = !(dtd > 0.0);
                    if (!bad) {
                        Mat<double, DIM>::inv(Jd, dtd, Jid);
                        #pragma unroll
                        for (int t = 0; t < DIM * DIM; ++t) Ji[t] = (float)Jid[t];
                        dt = (float)dtd;
                    } else {
                        dt = (float)dtd;
                    }
                    if (q == 0) atomicAdd(&a.status->flagged, 1u);
                }
            }
            if (bad) {
                record_detj(a.status, sd.cellid[cell], (float)dt);
                dt = Real(0);
                #pragma unroll
                for (int t = 0; t < DIM * DIM; ++t) Ji[t] = Real(0);
            }
            const Real s = sqrt(dt * w_s[q]);
            sq[q] = s;
            Real gradN[NB * DIM];  // unscaled physical gradients (neo-hooke needs them)
            #pragma unroll
            for (int i = 0; i < NB; ++i) {
                Real g[3] = {0, 0, 0};
                #pragma unroll
                for (int b = 0; b < DIM; ++b)
                    #pragma unroll
                    for (int c = 0; c < DIM; ++c) g[b] += dN_s[(q * NB + i) * DIM + c] * Ji[c * DIM + b];
                V4 v;
                v.x = g[0] * s;
                v.y = g[1] * s;
                v.z = DIM == 3 ? g[2] * s : Real(0);
                v.w = N_s[q * NB + i] * s;
                grad[q * NB + i] = v;
                if constexpr (PHYS == PHYS_NEO) {
                    #pragma unroll
                    for (int b = 0; b < DIM; ++b) gradN[i * DIM + b] = g[b];
                }
            }
            if (q == 0) {
                Real sc = Real(1);
                if (a.phys.scale_f) {
                    if constexpr (sizeof(Real) == 4) sc = a.phys.scale_f[sd.cellid[cell]];
                    else sc = a.phys.scale_d[sd.cellid[cell]];
                }
                if constexpr (PHYS == PHYS_ELASTIC) {
                    cellp[0] = (Real)a.phys.lam * sc;
                    cellp[1] = (Real)a.phys.mu * sc;
                } else {
                    cellp[0] = (Real)a.phys.p0 * sc;
                    cellp[1] = (Real)a.phys.p1;
                }
            }
            if constexpr (PHYS == PHYS_NEO) {
                // H = grad u = sum_i u_i (x) gradN_i (function_gradient, common_values.jl:217-227)
                Real H[9];
                #pragma unroll
                for (int t = 0; t < 9; ++t) H[t] = Real(0);
                const int32_t* en = sd.ents + (int64_t)cell * NB;
                #pragma unroll
                for (int i = 0; i < NB; ++i) {
                    const int64_t e3 = (int64_t)en[i] * 3;
                    Real ui[3];
                    #pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        if constexpr (sizeof(Real) == 4) ui[c] = a.phys.u_f[e3 + c];
                        else ui[c] = a.phys.u_d[e3 + c];
                    }
                    #pragma unroll
                    for (int c = 0; c < 3; ++c)
                        #pragma unroll
                        for (int J2 = 0; J2 < 3; ++J2) H[c * 3 + J2] += ui[c] * gradN[i * 3 + J2];
                }
                neo_hooke_point<Real>((Real)a.phys.p0, (Real)a.phys.p1, H, neo + q * NEO_EXTRA);
            }
        }
        __syncthreads();
        // ---------------- phase B: blocks of Ke into the owned columns ----------------
        const int it0 = a.wave_cell_items[w.cell_begin + s0];
        const int it1 = (s0 + nchunk < w.n_cells) ? a.wave_cell_items[w.cell_begin + s0 + nchunk] : w.item_begin + w.n_items;
        const int lane = tid % GS, grp = tid / GS;
        constexpr int NGRP = THREADS / GS;
        for (int it = it0 + grp; it < it1; it += NGRP) {
            const uint32_t word = a.items[it];
            const int slot = (int)(word >> (ITEM_J_BITS + ITEM_ENT_BITS)) - s0;
            const int j = (int)((word >> ITEM_ENT_BITS) & ((1u << ITEM_J_BITS) - 1));
            const int tent = (int)(word & ((1u << ITEM_ENT_BITS) - 1));
            const int i = lane;
            if (i >= NB) continue;
            const int cell = a.wave_cells[w.cell_begin + s0 + slot];
            const char* tb = sm.chunk + slot * TB;
            const V4* grad = (const V4*)tb;
            const Real* sq = (const Real*)(tb + NQ * NB * sizeof(V4));
            const Real* cellp = sq + NQ;
            const Real* neo = cellp + 4;
            const int4 et = sm.etab[tent];
            const int64_t rk = (int64_t)cell * NB * NB + j * NB + i;
            const int rank = sd.rank8 ? (sd.rank8[rk] == 255 ? -1 : (int)sd.rank8[rk])
                                      : (sd.rank16[rk] == 0xFFFF ? -1 : (int)sd.rank16[rk]);
            Real Kb[NC_MAX * NC_MAX];
            Real fe[NC_MAX];
            #pragma unroll
            for (int t = 0; t < NC_MAX * NC_MAX; ++t) Kb[t] = Real(0);
            #pragma unroll
            for (int t = 0; t < NC_MAX; ++t) fe[t] = Real(0);
            if constexpr (PHYS == PHYS_HEAT) {
                Real kk = 0, ff = 0;
                #pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    const V4 gi = grad[q * NB + i];
                    const V4 gj = grad[q * NB + j];
                    kk += gi.x * gj.x + gi.y * gj.y + (DIM == 3 ? gi.z * gj.z : Real(0));
                    ff += gj.w * sq[q];
                }
                Kb[0] = cellp[0] * kk;
                fe[0] = cellp[1] * ff;
            } else if constexpr (PHYS == PHYS_ELASTIC) {
                Real G[DIM * DIM];
                #pragma unroll
                for (int t = 0; t < DIM * DIM; ++t) G[t] = Real(0);
                Real ff = 0;
                #pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    const V4 gi = grad[q * NB + i];
                    const V4 gj = grad[q * NB + j];
                    const Real ai[3] = {gi.x, gi.y, gi.z}, aj[3] = {gj.x, gj.y, gj.z};
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x)
                        #pragma unroll
                        for (int y = 0; y < DIM; ++y) G[x * DIM + y] += ai[x] * aj[y];
                    ff += gj.w * sq[q];
                }
                const Real lam = cellp[0], mu = cellp[1];
                Real tr = 0;
                #pragma unroll
                for (int x = 0; x < DIM; ++x) tr += G[x * DIM + x];
                #pragma unroll
                for (int x = 0; x < DIM; ++x)
                    #pragma unroll
                    for (int y = 0; y < DIM; ++y) Kb[x * DIM + y] = lam * G[x * DIM + y] + mu * G[y * DIM + x] + (x == y ? mu * tr : Real(0));
                #pragma unroll
                for (int x = 0; x < DIM; ++x) fe[x] = ff * (Real)a.phys.body[x];
            } else {  // PHYS_NEO
                #pragma unroll 1
                for (int q = 0; q < NQ; ++q) {
                    const V4 gi = grad[q * NB + i];
                    const V4 gj = grad[q * NB + j];
                    const Real* nq_ = neo + q * NEO_EXTRA;
                    const Real ai[3] = {gi.x, gi.y, gi.z}, aj[3] = {gj.x, gj.y, gj.z};
                    Real Bi[3], Bj[3], tij = 0;
                    #pragma unroll
                    for (int x = 0; x < 3; ++x) {
                        Bi[x] = nq_[9 + x * 3] * ai[0] + nq_[9 + x * 3 + 1] * ai[1] + nq_[9 + x * 3 + 2] * ai[2];
                        Bj[x] = nq_[9 + x * 3] * aj[0] + nq_[9 + x * 3 + 1] * aj[1] + nq_[9 + x * 3 + 2] * aj[2];
                        tij += ai[x] * (nq_[x * 3] * aj[0] + nq_[x * 3 + 1] * aj[1] + nq_[x * 3 + 2] * aj[2]);
                    }
                    const Real c1 = nq_[18], c2x2 = nq_[19];
                    // K_ab += delta_ab giT.T.gj + c1 (B gi)_b (B gj)_a + 2c2 (B gi)_a (B gj)_b
                    #pragma unroll
                    for (int x = 0; x < 3; ++x)
                        #pragma unroll
                        for (int y = 0; y < 3; ++y)
                            Kb[x * 3 + y] += (x == y ? tij : Real(0)) + c1 * Bi[y] * Bj[x] + c2x2 * Bi[x] * Bj[y];
                    // residual: (gradN_j : P - N_j b) dV
                    const Real s = sq[q];
                    #pragma unroll
                    for (int x = 0; x < 3; ++x)
                        fe[x] += s * (nq_[20 + x * 3] * aj[0] + nq_[20 + x * 3 + 1] * aj[1] + nq_[20 + x * 3 + 2] * aj[2] -
                                      gj.w * (Real)a.phys.body[x]);
                }
            }
            // scatter into the accumulator: column entity (owned) = ent(j), row = ent(i)
            if (a.do_k) {
                if (rank < 0) {
                    #pragma unroll
                    for (int x = 0; x < NC_MAX; ++x)
                        #pragma unroll
                        for (int y = 0; y < NC_MAX; ++y)
                            if (x < nc && y < nc && Kb[x * NC_MAX + y] != Real(0))
                                record_miss(a.status, sd.cellid[cell], i * nc + x, j * nc + y);
                } else {
                    const int base = et.x + nc * rank;
                    if (nc == 1) {
                        acc_add(sm.acc[base], Kb[0]);
                    } else {
                        #pragma unroll
                        for (int y = 0; y < NC_MAX; ++y)
                            #pragma unroll
                            for (int x = 0; x < NC_MAX; ++x) acc_add(sm.acc[base + y * et.y + x], Kb[x * NC_MAX + y]);
                    }
                }
            }
            if (a.do_f && i == j) {
                #pragma unroll
                for (int x = 0; x < NC_MAX; ++x)
                    if (x < nc) acc_add(sm.facc[et.z + x], fe[x]);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// bounded wait on an mbarrier phase (TMA bulk copy completion)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, long long limit) {
    for (long long it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

// ---------------------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------------------
template <int K0, int Q0, int K1, int Q1, int K2, int Q2, int PHYS, typename Real>
__global__ void __launch_bounds__(THREADS, 1) tile_kernel(const KernelArgs a, const Real* __restrict__ shape_g, int shape_bytes,
                                                           int shape_off1, int shape_off2) {
    using Acc = typename AccT<Real>::type;
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ __align__(8) unsigned long long bar;
    Smem<Real> sm;
    char* p = smem_raw;
    sm.shape = (Real*)p;
    p += pad16(shape_bytes);
    sm.acc = (Acc*)p;
    p += pad16(a.acc_cap * (int)sizeof(Acc));
    sm.facc = (Acc*)p;
    p += pad16(a.ent_cap * a.nc * (int)sizeof(Acc));
    sm.etab = (int4*)p;
    p += a.ent_cap * (int)sizeof(int4);
    sm.chunk = p;

    const int tid = threadIdx.x;
    const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(&bar);
    // stage the reference tables with one TMA bulk copy
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_s), "r"(shape_bytes) : "memory");
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(sm.shape);
        asm volatile("cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                     "l"(shape_g), "r"(shape_bytes), "r"(bar_s)
                     : "memory");
    }
    __syncthreads();  // the initialised barrier is visible to every thread
    const TileDesc T = a.tiles[blockIdx.x];
    // entity table and zeroed (or loaded) accumulators
    {
        int base_ent = 0;
        for (int r = T.range_begin; r < T.range_end; ++r) {
            const RangeDesc R = a.ranges[r];
            for (int k = tid; k < R.n_ent; k += THREADS) {
                const int64_t n = (int64_t)R.ent0 + k;
                const int64_t c0 = a.colptr[a.nc * n] - 1;
                const int L = (int)(a.colptr[a.nc * n + 1] - a.colptr[a.nc * n]);
                sm.etab[base_ent + k] = make_int4(R.acc_base + (int)(c0 - R.nz0), L, (base_ent + k) * a.nc, 0);
            }
            if (a.fillzero) {
                for (int k = tid; k < R.nz_len; k += THREADS) acc_zero(sm.acc[R.acc_base + k]);
                for (int k = tid; k < R.n_ent * a.nc; k += THREADS) acc_zero(sm.facc[base_ent * a.nc + k]);
            } else {
                for (int k = tid; k < R.nz_len; k += THREADS) {
                    if (a.do_k) acc_set(sm.acc[R.acc_base + k], a.nzval[R.nz0 + k]);
                    else acc_zero(sm.acc[R.acc_base + k]);
                }
                for (int k = tid; k < R.n_ent * a.nc; k += THREADS) {
                    if (a.do_f) acc_set(sm.facc[base_ent * a.nc + k], a.f[(int64_t)R.ent0 * a.nc + k]);
                    else acc_zero(sm.facc[base_ent * a.nc + k]);
                }
            }
            base_ent += R.n_ent;
        }
    }
    // every thread waits for the table copy (bounded; a timeout skips the tile)
    const bool ok = mbar_wait(bar_s, 0, 1ll << 26);
    if (!ok) {
        if (tid == 0) atomicAdd(&a.status->timeout, 1u);
        return;
    }
    __syncthreads();
    for (int wi = T.wave_begin; wi < T.wave_end; ++wi) {
        const WaveDesc w = a.waves[wi];
        if (w.sub == 0) {
            process_wave<K0, Q0, PHYS, Real>(a, a.sub[0], sm.shape, w, sm);
        } else if constexpr (K1 >= 0) {
            if (w.sub == 1) {
                process_wave<K1, Q1, PHYS, Real>(a, a.sub[1], (const Real*)((const char*)sm.shape + shape_off1), w, sm);
            } else if constexpr (K2 >= 0) {
                process_wave<K2, Q2, PHYS, Real>(a, a.sub[2], (const Real*)((const char*)sm.shape + shape_off2), w, sm);
            }
        }
    }
    // write-out: every owned entry once, coalesced
    {
        int base_ent = 0;
        for (int r = T.range_begin; r < T.range_end; ++r) {
            const RangeDesc R = a.ranges[r];
            if (a.do_k)
                for (int k = tid; k < R.nz_len; k += THREADS) __stcs(a.nzval + R.nz0 + k, acc_value(sm.acc[R.acc_base + k]));
            if (a.do_f)
                for (int k = tid; k < R.n_ent * a.nc; k += THREADS)
                    __stcs(a.f + (int64_t)R.ent0 * a.nc + k, acc_value(sm.facc[base_ent * a.nc + k]));
            base_ent += R.n_ent;
        }
    }
}

}  // namespace fe
