// tile_kernel.cuh -- the owner-tile assembly kernel.
//
// One CTA assembles one tile: the nzval columns (and f entries) of a compact set of dof
// entities, written exactly once.
//   0. reference shape tables staged into shared memory with a TMA bulk copy
//      (cp.async.bulk + mbarrier); the tile's entity table; an empty contribution map.
//   1. for every subdomain segment and chunk of the tile's cells:
//      A. one thread per (cell, quadrature point): Jacobian from the node coordinates
//         (float hi+lo split, so cell-size differences keep FP32 relative accuracy), detJ,
//         J^-1 and sqrt(detJ w)-scaled physical gradients -> a shared-memory table, points
//         taken in pairs so one FFMA2 serves two points. Cells whose Jacobian condition
//         number exceeds a threshold are redone in FP64.
//      B. one lane group per cell, lane i = row base function, its table row kept in
//         registers: for every owned base function j of the cell, the nc x nc block
//         Ke[(i,:),(j,:)] (and fe_j on lane j) goes to its own staging slot
//         (entity(j), k, i), k = position of the cell among the entity's cells.
//   2. reduce: one lane per owned (entity, row entity) block sums its slots in k order
//      (cell order, compensated FP32 pair = FP64-class), rounds to FP64 and stores it.
// No atomics, no coloring, bitwise reproducible; the summation order of each entry is the
// reference's own cell order.
//
// Reference correspondence: step A is reinit!(cv, x) (src/FEValues/CellValues.jl:122-140,
// GeometryMapping.jl:124-130, FunctionValues.jl:186-192); step B is the element routine
// (heat_equation.jl:143-164, threaded_assembly.jl:105-119, hyperelasticity.jl:241-276);
// steps B+2 replace assemble! (src/assembler.jl:322-457) and fillzero!/addindex!
// (src/arrayutils.jl:100-152).
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

__device__ __forceinline__ double acc_value(float2 a) { return pair_to_double_fast(a.x, a.y); }
__device__ __forceinline__ double acc_value(double a) { return a; }
__device__ __forceinline__ void acc_zero(float2& a) { a = make_float2(0.f, 0.f); }
__device__ __forceinline__ void acc_init(float2& a, float x) { a = make_float2(x, 0.f); }
__device__ __forceinline__ void acc_init(double& a, double x) { a = x; }
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
    Real* stage;     // [stage_cap] block and f contributions, one slot each
    uint8_t* map;    // [map_cap] row function i of each (entity, row entity, k), 0xFF = none
    int4* emeta;     // [ent_cap] EntMeta of the owned entities
    int* eid;        // [ent_cap] their global ids
    unsigned long long* red_mask;  // [red_cap] which k hold a contribution, per owned block
    uint32_t* red;       // [red_cap] the tile's reduce order (prefetched)
    int4* col;           // [ent_cap] (colbase lo, colbase hi, column length, -) per owned entity
    uint32_t* items;     // [items_cap] the tile's items (prefetched)
    int* cells;          // [cells_cap] the tile's cells (subdomain-local ids)
    int* citems;         // [cells_cap] first item of each cell, relative to the tile
    int* conn;           // [cells_cap][ng_max] node ids of each cell
    Real* shape;     // staged reference tables of all subdomains
    char* chunk;     // per-chunk cell tables
};

// Shared-memory layout of a tile CTA, computed in one place for the kernel and the host.
struct SmemLayout {
    int shape, stage, map, emeta, eid, red_mask, red, col, items, cells, citems, conn, chunk;
};
__host__ __device__ inline int pad16i(int b) { return (b + 15) & ~15; }
__host__ __device__ inline SmemLayout smem_layout(const KernelArgs& a, int shape_bytes, int real_bytes) {
    SmemLayout L;
    int o = 0;
    L.shape = o; o += pad16i(shape_bytes);
    L.stage = o; o += pad16i(a.stage_cap * real_bytes);
    L.map = o; o += pad16i(a.map_cap);
    L.emeta = o; o += a.ent_cap * 16;
    L.eid = o; o += pad16i(a.ent_cap * 4);
    L.red_mask = o; o += pad16i(a.red_cap * 8);
    L.red = o; o += pad16i(a.red_cap * 4);
    L.col = o; o += a.ent_cap * 16;
    L.items = o; o += pad16i(a.items_cap * 4);
    L.cells = o; o += pad16i(a.cells_cap * 4);
    L.citems = o; o += pad16i(a.cells_cap * 4);
    L.conn = o; o += pad16i(a.cells_cap * a.ng_max * 4);
    L.chunk = o;
    return L;
}

template <typename Real> struct Pair;
template <> struct Pair<float> { using type = float2; };
template <> struct Pair<double> { using type = double2; };

// Packed multiply-add over a pair of quadrature points: one FFMA2 (sm_100+) for FP32.
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ double2 pfma(double2 a, double2 b, double2 c) {
    return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
template <typename P> __device__ __forceinline__ P pzero();
template <> __device__ __forceinline__ float2 pzero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double2 pzero<double2>() { return make_double2(0.0, 0.0); }

// Cell table layout (one cell of a chunk), quadrature points taken in pairs (q0 = 2p, q1 = 2p+1;
// an odd count is padded with a zero-weight point):
//   grad[NQP][NB][8] : (gx0, gx1, gy0, gy1, gz0, gz1, n0, n1), g = sqrt(detJ w) gradN, n = sqrt(detJ w) N
//   sq[NQP][2]       : sqrt(detJ w) per point
//   cellp[4]         : per-cell material values
//   neo[NQ][NEO_EXTRA] (Neo-Hooke only)
template <int K, int NQ, int PHYS, typename Real>
struct CellTable {
    static constexpr int NB = ElemT<K>::NB;
    static constexpr int NQP = (NQ + 1) / 2;
    static constexpr int GRAD = NQP * NB * 8;
    static constexpr int SQ = NQP * 2;
    static constexpr int NEO = PHYS == PHYS_NEO ? NQ * NEO_EXTRA : 0;
    static constexpr int REALS = GRAD + SQ + 4 + NEO;
    static constexpr int BYTES = (REALS * (int)sizeof(Real) + 15) & ~15;
};

template <int K, int NQ, int PHYS, typename Real>
__host__ __device__ constexpr int cell_table_bytes() {
    return CellTable<K, NQ, PHYS, Real>::BYTES;
}

// shape table block per subdomain: w[NQ], N[NQ][NB], dN[NQ][NB][DIM], dM[NQ][NG][DIM],
// each padded to a multiple of 16 bytes
__host__ __device__ inline int pad16(int bytes) { return (bytes + 15) & ~15; }
template <typename Real>
__host__ __device__ inline int shape_block_bytes(int nq, int nb, int ng, int dim) {
    return pad16(nq * (int)sizeof(Real)) + pad16(nq * nb * (int)sizeof(Real)) + pad16(nq * nb * dim * (int)sizeof(Real)) +
           pad16(nq * ng * dim * (int)sizeof(Real));
}

// ---------------------------------------------------------------------------------------
// phase A: geometry of one cell at one pair of quadrature points (q0 = 2p, q1 = 2p + 1)
// ---------------------------------------------------------------------------------------
template <int K, int NQ, int PHYS, typename Real>
__device__ __forceinline__ void geometry_pair(const KernelArgs& a, const SubDev& sd, const Real* w_s, const Real* N_s,
                                              const Real* dN_s, const Real* dM_s, int cell, const int* cn, int p, Real* tb) {
    using E = ElemT<K>;
    using CT = CellTable<K, NQ, PHYS, Real>;
    using P = typename Pair<Real>::type;
    constexpr int NB = E::NB, NG = E::NG, DIM = E::DIM;
    Real* grad = tb;
    Real* sq = tb + CT::GRAD;
    Real* cellp = sq + CT::SQ;
    Real* neo = cellp + 4;
    const int nq = (2 * p + 1 < NQ) ? 2 : 1;
    // node offsets from node 0 (float hi/lo split keeps them accurate to FP32 relative)
    Real off[NG][DIM];
    const int n0 = cn[0];
    if constexpr (sizeof(Real) == 4) {
        float h0[DIM], l0[DIM];
        #pragma unroll
        for (int x = 0; x < DIM; ++x) { h0[x] = __ldg(a.xh[x] + n0); l0[x] = __ldg(a.xl[x] + n0); }
        #pragma unroll
        for (int k = 1; k < NG; ++k) {
            const int nk = cn[k];
            #pragma unroll
            for (int x = 0; x < DIM; ++x) off[k][x] = (__ldg(a.xh[x] + nk) - h0[x]) + (__ldg(a.xl[x] + nk) - l0[x]);
        }
    } else {
        double x0[DIM];
        #pragma unroll
        for (int x = 0; x < DIM; ++x) x0[x] = a.xd[(int64_t)n0 * a.dim + x];
        #pragma unroll
        for (int k = 1; k < NG; ++k) {
            const int nk = cn[k];
            #pragma unroll
            for (int x = 0; x < DIM; ++x) off[k][x] = a.xd[(int64_t)nk * a.dim + x] - x0[x];
        }
    }
    Real Ji[2][DIM * DIM], sc[2];
    #pragma unroll
    for (int h = 0; h < 2; ++h) {
        sc[h] = Real(0);
        #pragma unroll
        for (int t = 0; t < DIM * DIM; ++t) Ji[h][t] = Real(0);
        if (h >= nq) continue;
        const int q = 2 * p + h;
        Real J[DIM * DIM];
        #pragma unroll
        for (int t = 0; t < DIM * DIM; ++t) J[t] = Real(0);
        #pragma unroll
        for (int k = 1; k < NG; ++k)
            #pragma unroll
            for (int x = 0; x < DIM; ++x)
                #pragma unroll
                for (int b = 0; b < DIM; ++b) J[x * DIM + b] += off[k][x] * dM_s[(q * NG + k) * DIM + b];
        Real dt = Mat<Real, DIM>::det(J);
        bool bad = !(dt > Real(0));
        if (!bad) Mat<Real, DIM>::inv(J, dt, Ji[h]);
        if constexpr (sizeof(Real) == 4) {
            // FP64 Jacobian for flagged cells: Frobenius condition estimate
            float nJ = 0, nJi = 0;
            if (!bad) {
                #pragma unroll
                for (int t = 0; t < DIM * DIM; ++t) { nJ += J[t] * J[t]; nJi += Ji[h][t] * Ji[h][t]; }
            }
            if (bad || nJ * nJi > a.phys.cond_threshold * a.phys.cond_threshold * DIM * DIM) {
                double Jd[DIM * DIM], Jid[DIM * DIM];
                #pragma unroll
                for (int t = 0; t < DIM * DIM; ++t) Jd[t] = 0.0;
                double x0[DIM];
                #pragma unroll
                for (int x = 0; x < DIM; ++x) x0[x] = a.xd[(int64_t)n0 * a.dim + x];
                for (int k = 1; k < NG; ++k) {
                    const int nk = cn[k];
                    for (int x = 0; x < DIM; ++x) {
                        const double o = a.xd[(int64_t)nk * a.dim + x] - x0[x];
                        for (int b = 0; b < DIM; ++b) Jd[x * DIM + b] += o * sd.dM_d[(q * NG + k) * DIM + b];
                    }
                }
                const double dtd = Mat<double, DIM>::det(Jd);
                bad = !(dtd > 0.0);
                if (!bad) {
                    Mat<double, DIM>::inv(Jd, dtd, Jid);
                    #pragma unroll
                    for (int t = 0; t < DIM * DIM; ++t) Ji[h][t] = (float)Jid[t];
                }
                dt = (float)dtd;
                if (q == 0) atomicAdd(&a.status->flagged, 1u);
            }
        }
        if (bad) {
            record_detj(a.status, sd.cellid[cell], (float)dt);
            dt = Real(0);
            #pragma unroll
            for (int t = 0; t < DIM * DIM; ++t) Ji[h][t] = Real(0);
        }
        sc[h] = sqrt(dt * w_s[q]);
    }
    *(P*)(sq + 2 * p) = P{sc[0], sc[1]};
    Real H[2][9];
    #pragma unroll
    for (int h = 0; h < 2; ++h)
        #pragma unroll
        for (int t = 0; t < 9; ++t) H[h][t] = Real(0);
    #pragma unroll
    for (int i = 0; i < NB; ++i) {
        Real g[2][3];
        Real nn[2];
        #pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int q = min(2 * p + h, NQ - 1);
            #pragma unroll
            for (int b = 0; b < 3; ++b) g[h][b] = Real(0);
            #pragma unroll
            for (int b = 0; b < DIM; ++b)
                #pragma unroll
                for (int c = 0; c < DIM; ++c) g[h][b] += dN_s[(q * NB + i) * DIM + c] * Ji[h][c * DIM + b];
            nn[h] = N_s[q * NB + i];
        }
        if constexpr (PHYS == PHYS_NEO) {
            const int64_t e3 = (int64_t)sd.ents[(int64_t)cell * NB + i] * 3;
            #pragma unroll
            for (int c = 0; c < 3; ++c) {
                Real uc;
                if constexpr (sizeof(Real) == 4) uc = a.phys.u_f[e3 + c];
                else uc = a.phys.u_d[e3 + c];
                #pragma unroll
                for (int h = 0; h < 2; ++h)
                    #pragma unroll
                    for (int J2 = 0; J2 < 3; ++J2) H[h][c * 3 + J2] += uc * g[h][J2];
            }
        }
        P* o = (P*)(grad + (p * NB + i) * 8);
        o[0] = P{g[0][0] * sc[0], g[1][0] * sc[1]};
        o[1] = P{g[0][1] * sc[0], g[1][1] * sc[1]};
        o[2] = P{g[0][2] * sc[0], g[1][2] * sc[1]};
        o[3] = P{nn[0] * sc[0], nn[1] * sc[1]};
    }
    if (p == 0) {
        Real scale = Real(1);
        if (a.phys.scale_f) {
            if constexpr (sizeof(Real) == 4) scale = a.phys.scale_f[sd.cellid[cell]];
            else scale = a.phys.scale_d[sd.cellid[cell]];
        }
        if constexpr (PHYS == PHYS_ELASTIC) {
            cellp[0] = (Real)a.phys.lam * scale;
            cellp[1] = (Real)a.phys.mu * scale;
        } else {
            cellp[0] = (Real)a.phys.p0 * scale;
            cellp[1] = (Real)a.phys.p1;
        }
    }
    if constexpr (PHYS == PHYS_NEO) {
        #pragma unroll
        for (int h = 0; h < 2; ++h)
            if (h < nq) neo_hooke_point<Real>((Real)a.phys.p0, (Real)a.phys.p1, H[h], neo + (2 * p + h) * NEO_EXTRA);
    }
}

// ---------------------------------------------------------------------------------------
// phase B: the blocks of one cell into its owned columns; lane i = row base function
// ---------------------------------------------------------------------------------------
template <int K, int NQ, int PHYS, typename Real>
__device__ __forceinline__ void cell_blocks(const KernelArgs& a, const SubDev& sd, const Smem<Real>& sm, const Real* tb,
                                            int cell, int i, int it0, int it1) {
    using E = ElemT<K>;
    using CT = CellTable<K, NQ, PHYS, Real>;
    using P = typename Pair<Real>::type;
    constexpr int NB = E::NB, DIM = E::DIM, NQP = CT::NQP;
    constexpr int NC_MAX = DIM;
    constexpr bool CACHE = NQP <= 4;  // keep the row function's table in registers
    const int nc = a.nc;
    const Real* grad = tb;
    const Real* sq = tb + CT::GRAD;
    const Real* cellp = sq + CT::SQ;
    const Real* neo = cellp + 4;
    P gi[CACHE ? NQP : 1][4];
    if constexpr (CACHE) {
        #pragma unroll
        for (int p = 0; p < NQP; ++p)
            #pragma unroll
            for (int c = 0; c < 4; ++c) gi[p][c] = *(const P*)(grad + (p * NB + i) * 8 + 2 * c);
    }
    // this lane's rank row: the rank of entity(i) in the columns of every entity(j) of the cell
    constexpr int RW8 = (NB + 7) / 8, RW16 = (NB + 3) / 4;
    unsigned long long rrow[RW8 > RW16 ? RW8 : RW16];
    if (sd.rank8) {
        const unsigned long long* rp = (const unsigned long long*)(sd.rank8 + ((int64_t)cell * NB + i) * (8 * RW8));
        #pragma unroll
        for (int t = 0; t < RW8; ++t) rrow[t] = __ldg(rp + t);
    } else {
        const unsigned long long* rp = (const unsigned long long*)(sd.rank16 + ((int64_t)cell * NB + i) * (4 * RW16));
        #pragma unroll
        for (int t = 0; t < RW16; ++t) rrow[t] = __ldg(rp + t);
    }
    for (int it = it0; it < it1; ++it) {
        const uint32_t word = sm.items[it];
        const int j = (int)(word & ((1u << ITEM_J_BITS) - 1));
        const int tent = (int)((word >> ITEM_J_BITS) & ((1u << ITEM_ENT_BITS) - 1));
        const int kk = (int)(word >> (ITEM_J_BITS + ITEM_ENT_BITS));
        int rank;
        if (sd.rank8) {
            unsigned long long w = rrow[0];
            #pragma unroll
            for (int t = 1; t < RW8; ++t)
                if (t == (j >> 3)) w = rrow[t];
            const int v = (int)((w >> ((j & 7) * 8)) & 0xFF);
            rank = v == 0xFF ? -1 : v;
        } else {
            unsigned long long w = rrow[0];
            #pragma unroll
            for (int t = 1; t < RW16; ++t)
                if (t == (j >> 2)) w = rrow[t];
            const int v = (int)((w >> ((j & 3) * 16)) & 0xFFFF);
            rank = v == 0xFFFF ? -1 : v;
        }
        Real Kb[NC_MAX * NC_MAX];
        Real fe[NC_MAX];
        #pragma unroll
        for (int t = 0; t < NC_MAX * NC_MAX; ++t) Kb[t] = Real(0);
        #pragma unroll
        for (int t = 0; t < NC_MAX; ++t) fe[t] = Real(0);
        if constexpr (PHYS == PHYS_HEAT || PHYS == PHYS_ELASTIC) {
            P G[DIM][DIM];
            P ff = pzero<P>();
            #pragma unroll
            for (int x = 0; x < DIM; ++x)
                #pragma unroll
                for (int y = 0; y < DIM; ++y) G[x][y] = pzero<P>();
            #pragma unroll
            for (int p = 0; p < NQP; ++p) {
                P ri[4], rj[4];
                #pragma unroll
                for (int c = 0; c < 4; ++c) {
                    if constexpr (CACHE) ri[c] = gi[p][c];
                    else ri[c] = *(const P*)(grad + (p * NB + i) * 8 + 2 * c);
                    rj[c] = *(const P*)(grad + (p * NB + j) * 8 + 2 * c);
                }
                if constexpr (PHYS == PHYS_HEAT) {
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x) G[0][0] = pfma(ri[x], rj[x], G[0][0]);
                } else {
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x)
                        #pragma unroll
                        for (int y = 0; y < DIM; ++y) G[x][y] = pfma(ri[x], rj[y], G[x][y]);
                }
                ff = pfma(*(const P*)(sq + 2 * p), rj[3], ff);
            }
            if constexpr (PHYS == PHYS_HEAT) {
                Kb[0] = cellp[0] * (G[0][0].x + G[0][0].y);
                fe[0] = cellp[1] * (ff.x + ff.y);
            } else {
                Real g[DIM][DIM];
                #pragma unroll
                for (int x = 0; x < DIM; ++x)
                    #pragma unroll
                    for (int y = 0; y < DIM; ++y) g[x][y] = G[x][y].x + G[x][y].y;
                const Real lam = cellp[0], mu = cellp[1];
                Real tr = 0;
                #pragma unroll
                for (int x = 0; x < DIM; ++x) tr += g[x][x];
                #pragma unroll
                for (int x = 0; x < DIM; ++x)
                    #pragma unroll
                    for (int y = 0; y < DIM; ++y) Kb[x * DIM + y] = lam * g[x][y] + mu * g[y][x] + (x == y ? mu * tr : Real(0));
                const Real fs = ff.x + ff.y;
                #pragma unroll
                for (int x = 0; x < DIM; ++x) fe[x] = fs * (Real)a.phys.body[x];
            }
        } else {  // PHYS_NEO: per point, scalar
            #pragma unroll 1
            for (int q = 0; q < NQ; ++q) {
                const int p = q >> 1, h = q & 1;
                const Real* gio = grad + (p * NB + i) * 8 + h;
                const Real* gjo = grad + (p * NB + j) * 8 + h;
                const Real ai[3] = {gio[0], gio[2], gio[4]}, aj[3] = {gjo[0], gjo[2], gjo[4]};
                const Real nj = gjo[6];
                const Real* nq_ = neo + q * NEO_EXTRA;
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
                const Real s = sq[2 * p + h];
                #pragma unroll
                for (int x = 0; x < 3; ++x)
                    fe[x] += s * (nq_[20 + x * 3] * aj[0] + nq_[20 + x * 3 + 1] * aj[1] + nq_[20 + x * 3 + 2] * aj[2] -
                                  nj * (Real)a.phys.body[x]);
            }
        }
        // one staging slot per (entity, k, i): no two lanes of the CTA ever write the same one
        const int4 m = sm.emeta[tent];
        const int kcnt = m.w & 0xFF;
        if (a.do_k) {
            if (rank < 0) {
                #pragma unroll
                for (int x = 0; x < NC_MAX; ++x)
                    #pragma unroll
                    for (int y = 0; y < NC_MAX; ++y)
                        if (x < nc && y < nc && Kb[x * NC_MAX + y] != Real(0))
                            record_miss(a.status, sd.cellid[cell], i * nc + x, j * nc + y);
            } else {
                Real* dst = sm.stage + m.x + (kk * a.nb_max + i) * a.bs;
                if (nc == 1) {
                    dst[0] = Kb[0];
                } else {
                    // column-major (b outer) so the reduce step reads in output order; an
                    // odd count is padded with a zero so slots are pairs
                    Real col[NC_MAX * NC_MAX + 1];
                    #pragma unroll
                    for (int y = 0; y < NC_MAX; ++y)
                        #pragma unroll
                        for (int x = 0; x < NC_MAX; ++x) col[y * NC_MAX + x] = Kb[x * NC_MAX + y];
                    col[NC_MAX * NC_MAX] = Real(0);
                    // nc is 1 (scalar field) or the dimension (vector field): the host checks it
                    #pragma unroll
                    for (int t = 0; t < (NC_MAX * NC_MAX + 1) / 2; ++t) ((P*)dst)[t] = P{col[2 * t], col[2 * t + 1]};
                }
                sm.map[m.y + rank * kcnt + kk] = (uint8_t)i;
                atomicOr(&sm.red_mask[m.z + rank], 1ull << kk);
            }
        }
        if (a.do_f && i == j) {
            Real* dst = sm.stage + m.x + kcnt * a.nb_max * a.bs + kk * nc;
            #pragma unroll
            for (int x = 0; x < NC_MAX; ++x)
                if (x < nc) dst[x] = fe[x];
        }
    }
}

// ---------------------------------------------------------------------------------------
// the cells of one subdomain in a tile, in chunks that fit the table memory
// ---------------------------------------------------------------------------------------
template <int K, int NQ, int PHYS, typename Real>
__device__ __forceinline__ void process_segment(const KernelArgs& a, const SubDev& sd, const Real* shp, const SegDesc& g,
                                                const TileDesc& T, const Smem<Real>& sm) {
    using E = ElemT<K>;
    using CT = CellTable<K, NQ, PHYS, Real>;
    constexpr int NB = E::NB, DIM = E::DIM, GS = E::GS;
    const Real* w_s = shp;
    const Real* N_s = (const Real*)((const char*)w_s + pad16(NQ * sizeof(Real)));
    const Real* dN_s = (const Real*)((const char*)N_s + pad16(NQ * NB * sizeof(Real)));
    const Real* dM_s = (const Real*)((const char*)dN_s + pad16(NQ * NB * DIM * sizeof(Real)));
    const int tid = threadIdx.x;
    const int tb0 = g.cell_begin - T.cell_begin, item_end = g.item_end - T.item_begin;
    // one lane group per cell (round robin), each with a private table buffer: the group
    // computes its cell's geometry (lanes = quadrature point pairs), syncs within the warp,
    // then its lanes (= row base functions) compute and stage the blocks
    constexpr int NQP = CT::NQP;
    const int ngrp = a.groups[g.sub];  // <= THREADS / GS, bounded by the table memory
    const int lane = tid % GS, grp = tid / GS;
    const unsigned gmask = GS >= 32 ? 0xFFFFFFFFu : (((1u << GS) - 1u) << ((tid & 31) / GS * GS));
    Real* tb = (Real*)(sm.chunk + grp * CT::BYTES);
    for (int c = grp < ngrp ? grp : g.n_cells; c < g.n_cells; c += ngrp) {
        const int ts = tb0 + c;
        const int cell = sm.cells[ts];
        for (int pp = lane; pp < NQP; pp += GS) geometry_pair<K, NQ, PHYS, Real>(a, sd, w_s, N_s, dN_s, dM_s, cell, sm.conn + ts * a.ng_max, pp, tb);
        __syncwarp(gmask);
        if (lane < NB) {
            const int it0 = sm.citems[ts];
            const int it1 = (c + 1 < g.n_cells) ? sm.citems[ts + 1] : item_end;
            cell_blocks<K, NQ, PHYS, Real>(a, sd, sm, tb, cell, lane, it0, it1);
        }
        __syncwarp(gmask);  // the next cell overwrites the table
    }
}

// ---------------------------------------------------------------------------------------
// reduce: one lane per owned (entity n, row entity r) block. The block's contributions are
// summed in cell order (k), compensated, rounded to FP64 and stored: nc columns of nc rows.
// ---------------------------------------------------------------------------------------
// Packed compensated sum over two entries (FP32 pairs); exact TwoSum per component.
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ void acc_add2(float2& hi, float2& lo, float2 x) {
    const float2 s = __fadd2_rn(hi, x);
    const float2 bb = fsub2(s, hi);
    const float2 e = __fadd2_rn(fsub2(hi, fsub2(s, bb)), fsub2(x, bb));
    hi = s;
    lo = __fadd2_rn(lo, e);
}

// One lane per owned (entity, row entity) block, in the plan's order (most contributions
// first, so the lanes of a warp run loops of equal length; the lane does not change any
// value). The block's slots are summed in k order (cell order) and the block is stored.
template <int NC, typename Real>
__device__ __forceinline__ void reduce_tile(const KernelArgs& a, const TileDesc& T, const Smem<Real>& sm) {
    constexpr int NCC = NC * NC, BS = (NCC + 1) & ~1, NP = BS / 2;
    using P = typename Pair<Real>::type;
    for (int pos = threadIdx.x; pos < T.n_red; pos += THREADS) {
        const uint32_t key = sm.red[pos];
        const int e = (int)(key >> 22), r = (int)(key & ((1u << 22) - 1));
        const int4 m = sm.emeta[e];
        const int kcnt = m.w & 0xFF;
        unsigned long long mask = sm.red_mask[m.z + r];
        const int4 cl = sm.col[e];
        const int64_t c0 = (int64_t)(uint32_t)cl.x | ((int64_t)cl.y << 32);
        const int64_t L = cl.z;
        const uint8_t* mp = sm.map + m.y + r * kcnt;
        double out[NCC];
        if constexpr (sizeof(Real) == 4) {
            float2 hi[NP], lo[NP];
            #pragma unroll
            for (int t = 0; t < NP; ++t) { hi[t] = make_float2(0.f, 0.f); lo[t] = make_float2(0.f, 0.f); }
            if (!a.fillzero) {
                float hv[BS], lv[BS];
                #pragma unroll
                for (int t = 0; t < BS; ++t) { hv[t] = 0.f; lv[t] = 0.f; }
                #pragma unroll
                for (int b = 0; b < NC; ++b)
                    #pragma unroll
                    for (int x = 0; x < NC; ++x) {
                        float2 q;
                        acc_set(q, a.nzval[c0 + b * L + NC * r + x]);
                        hv[b * NC + x] = q.x;
                        lv[b * NC + x] = q.y;
                    }
                #pragma unroll
                for (int t = 0; t < NP; ++t) { hi[t] = make_float2(hv[2 * t], hv[2 * t + 1]); lo[t] = make_float2(lv[2 * t], lv[2 * t + 1]); }
            } else if (mask) {
                const int k = __ffsll((long long)mask) - 1;
                mask &= mask - 1;
                const float2* v = (const float2*)(sm.stage + m.x + (k * a.nb_max + mp[k]) * BS);
                #pragma unroll
                for (int t = 0; t < NP; ++t) hi[t] = v[t];
            }
            while (mask) {
                const int k = __ffsll((long long)mask) - 1;
                mask &= mask - 1;
                const float2* v = (const float2*)(sm.stage + m.x + (k * a.nb_max + mp[k]) * BS);
                #pragma unroll
                for (int t = 0; t < NP; ++t) acc_add2(hi[t], lo[t], v[t]);
            }
            #pragma unroll
            for (int t = 0; t < NP; ++t) {
                out[2 * t] = pair_to_double_fast(hi[t].x, lo[t].x);
                if (2 * t + 1 < NCC) out[2 * t + 1] = pair_to_double_fast(hi[t].y, lo[t].y);
            }
        } else {
            double acc[NCC];
            #pragma unroll
            for (int t = 0; t < NCC; ++t) acc[t] = 0.0;
            if (!a.fillzero) {
                #pragma unroll
                for (int b = 0; b < NC; ++b)
                    #pragma unroll
                    for (int x = 0; x < NC; ++x) acc[b * NC + x] = a.nzval[c0 + b * L + NC * r + x];
            }
            while (mask) {
                const int k = __ffsll((long long)mask) - 1;
                mask &= mask - 1;
                const Real* v = sm.stage + m.x + (k * a.nb_max + mp[k]) * BS;
                #pragma unroll
                for (int t = 0; t < NCC; ++t) acc[t] += v[t];
            }
            #pragma unroll
            for (int t = 0; t < NCC; ++t) out[t] = acc[t];
        }
        #pragma unroll
        for (int b = 0; b < NC; ++b)
            #pragma unroll
            for (int x = 0; x < NC; ++x) __stcs(a.nzval + c0 + b * L + NC * r + x, out[b * NC + x]);
    }
}

template <typename Real>
__device__ __forceinline__ void reduce_f(const KernelArgs& a, const TileDesc& T, const Smem<Real>& sm) {
    using Acc = typename AccT<Real>::type;
    const int nc = a.nc;
    for (int idx = threadIdx.x; idx < T.n_ent * nc; idx += THREADS) {
        const int e = idx / nc, x = idx - e * nc;
        const int4 m = sm.emeta[e];
        const int kcnt = m.w & 0xFF;
        const int64_t gi = (int64_t)sm.eid[e] * nc + x;
        Acc acc;
        acc_zero(acc);
        if (!a.fillzero) acc_set(acc, a.f[gi]);
        const Real* v = sm.stage + m.x + kcnt * a.nb_max * a.bs + x;
        for (int k = 0; k < kcnt; ++k) acc_add(acc, v[k * nc]);
        __stcs(a.f + gi, acc_value(acc));
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
__global__ void __launch_bounds__(THREADS, 2) tile_kernel(const KernelArgs a, const Real* __restrict__ shape_g, int shape_bytes,
                                                           int shape_off1, int shape_off2) {
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ __align__(8) unsigned long long bar;
    Smem<Real> sm;
    const SmemLayout lay = smem_layout(a, shape_bytes, (int)sizeof(Real));
    {
        // the host sized the allocation from the same layout; refuse to run past it
        uint32_t dyn;
        asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
        if ((uint32_t)(lay.chunk + a.chunk_bytes) > dyn) {
            if (threadIdx.x == 0) atomicAdd(&a.status->timeout, 1u);
            return;
        }
    }
    sm.shape = (Real*)(smem_raw + lay.shape);
    sm.stage = (Real*)(smem_raw + lay.stage);
    sm.map = (uint8_t*)(smem_raw + lay.map);
    sm.emeta = (int4*)(smem_raw + lay.emeta);
    sm.eid = (int*)(smem_raw + lay.eid);
    sm.red_mask = (unsigned long long*)(smem_raw + lay.red_mask);
    sm.red = (uint32_t*)(smem_raw + lay.red);
    sm.col = (int4*)(smem_raw + lay.col);
    sm.items = (uint32_t*)(smem_raw + lay.items);
    sm.cells = (int*)(smem_raw + lay.cells);
    sm.citems = (int*)(smem_raw + lay.citems);
    sm.conn = (int*)(smem_raw + lay.conn);
    sm.chunk = smem_raw + lay.chunk;

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
    // one burst of independent loads: owned entities with their column bases, the reduce
    // order, the tile's cells, items and connectivity
    for (int e = tid; e < T.n_ent; e += THREADS) {
        sm.emeta[e] = reinterpret_cast<const int4*>(a.emeta)[T.ent_begin + e];
        const int n = a.eids[T.ent_begin + e];
        sm.eid[e] = n;
        const int64_t c0 = a.colptr[(int64_t)a.nc * n] - 1;
        const int L = (int)(a.colptr[(int64_t)a.nc * n + 1] - a.colptr[(int64_t)a.nc * n]);
        sm.col[e] = make_int4((int)(c0 & 0xFFFFFFFF), (int)(c0 >> 32), L, 0);
    }
    for (int k = tid; k < T.n_red; k += THREADS) sm.red[k] = a.red_list[T.red_begin + k];
    for (int k = tid; k < T.n_items; k += THREADS) sm.items[k] = a.items[T.item_begin + k];
    for (int k = tid; k < T.n_cells; k += THREADS) {
        sm.cells[k] = a.tile_cells[T.cell_begin + k];
        sm.citems[k] = a.cell_items[T.cell_begin + k] - T.item_begin;
    }
    for (int gi = T.seg_begin; gi < T.seg_end; ++gi) {
        const SegDesc g = a.segs[gi];
        const SubDev& sd = a.sub[g.sub];
        const int ng = sd.ng, t0 = g.cell_begin - T.cell_begin;
        for (int idx = tid; idx < g.n_cells * ng; idx += THREADS) {
            const int c = idx / ng, k = idx - c * ng;
            const int cell = a.tile_cells[g.cell_begin + c];
            sm.conn[(t0 + c) * a.ng_max + k] = sd.conn[(int64_t)cell * ng + k];
        }
    }
    {
        int4* mp = (int4*)sm.map;
        const int n16 = (T.map_bytes + 15) >> 4;
        for (int k = tid; k < n16; k += THREADS) mp[k] = make_int4(-1, -1, -1, -1);
        for (int k = tid; k < T.n_red; k += THREADS) sm.red_mask[k] = 0ull;
    }
    // every thread waits for the table copy (bounded; a timeout skips the tile)
    const bool ok = mbar_wait(bar_s, 0, 1ll << 26);
    if (!ok) {
        if (tid == 0) atomicAdd(&a.status->timeout, 1u);
        return;
    }
    __syncthreads();
    for (int gi = T.seg_begin; gi < T.seg_end; ++gi) {
        const SegDesc g = a.segs[gi];
        if (gi > T.seg_begin) __syncthreads();  // table buffers are laid out per element kind
        if (g.sub == 0) {
            process_segment<K0, Q0, PHYS, Real>(a, a.sub[0], sm.shape, g, T, sm);
        } else if constexpr (K1 >= 0) {
            if (g.sub == 1) {
                process_segment<K1, Q1, PHYS, Real>(a, a.sub[1], (const Real*)((const char*)sm.shape + shape_off1), g, T, sm);
            } else if constexpr (K2 >= 0) {
                process_segment<K2, Q2, PHYS, Real>(a, a.sub[2], (const Real*)((const char*)sm.shape + shape_off2), g, T, sm);
            }
        }
    }
    __syncthreads();  // all staging slots and masks written
    if (a.do_k) {
        if (a.nc == 3) reduce_tile<3, Real>(a, T, sm);
        else if (a.nc == 2) reduce_tile<2, Real>(a, T, sm);
        else reduce_tile<1, Real>(a, T, sm);
    }
    if (a.do_f) reduce_f<Real>(a, T, sm);
}

}  // namespace fe
