// tile_kernel.cuh -- the owner-tile assembly kernel.
//
// A persistent CTA assembles tiles t = blockIdx.x, + gridDim.x, ...: each tile is the nzval
// columns (and f entries) of a compact set of dof entities, written exactly once. A tile's
// plan data is one contiguous record (common.h), so the CTA streams it:
//   pipeline. While tile t is computed, the record of tile t + 2G arrives by one TMA bulk
//      copy (cp.async.bulk + mbarrier) and the node coordinates of tile t + G are gathered
//      into shared memory (cp.async); the reference shape tables are copied once per CTA.
//   1. for every subdomain segment of the tile, one lane group per cell:
//      A. lane q = quadrature point: Jacobian from the node coordinates (float hi+lo split,
//         so cell-size differences keep FP32 relative accuracy), detJ, J^-1 and
//         sqrt(detJ w)-scaled physical gradients -> the group's shared-memory table, points
//         paired so one FFMA2 serves two points. Cells whose Jacobian condition number
//         exceeds a threshold are redone in FP64.
//      B. lane i = row base function, its table row kept in registers: for every owned
//         base function j of the cell, the nc x nc block Ke[(i,:),(j,:)] (and fe_j on lane
//         j) goes to the staging slot the plan assigned to it.
//   2. reduce: one lane per owned (entity, row entity) block sums its consecutive slots
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

#include <type_traits>

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

static_assert(ElemT<KIND_TRI3>::GS == GROUP_LANES[KIND_TRI3] && ElemT<KIND_QUAD4>::GS == GROUP_LANES[KIND_QUAD4] &&
                  ElemT<KIND_TET4>::GS == GROUP_LANES[KIND_TET4] && ElemT<KIND_HEX8>::GS == GROUP_LANES[KIND_HEX8] &&
                  ElemT<KIND_WEDGE6>::GS == GROUP_LANES[KIND_WEDGE6] && ElemT<KIND_HEX27>::GS == GROUP_LANES[KIND_HEX27] &&
                  ElemT<KIND_QUAD9>::GS == GROUP_LANES[KIND_QUAD9],
              "lane groups agree with the planner");

constexpr int PHYS_HEAT = 1, PHYS_ELASTIC = 2, PHYS_NEO = 3;
constexpr int NEO_POINT = 29;  // neo_hooke_point output: T = S + c1 C^-1 (9), B = F^-T (9), c1, 2c2, P (9)
// Neo-Hooke cell-table entries per quadrature-point pair (values of the two points
// interleaved): T's six distinct entries (T is symmetric: S and C^-1 are), c1, 2c2, then
// s P (9) for the residual
constexpr int NEO_PAIR = 34;
constexpr int NEO_T = 0, NEO_C1 = 12, NEO_C2 = 14, NEO_SP = 16;
constexpr int THREADS = CTA_THREADS;

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

__device__ __forceinline__ double acc_value(float2 a) {
    bool rare = false;
    const double v = pair1_to_double(a.x, a.y, rare);
    return rare ? pair_to_double(a.x, a.y) : v;
}
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
    static __device__ __forceinline__ void adj(const R* J, R* A) {  // J^-1 = A / det
        A[0] = J[4] * J[8] - J[5] * J[7];
        A[1] = -(J[1] * J[8] - J[2] * J[7]);
        A[2] = J[1] * J[5] - J[2] * J[4];
        A[3] = -(J[3] * J[8] - J[5] * J[6]);
        A[4] = J[0] * J[8] - J[2] * J[6];
        A[5] = -(J[0] * J[5] - J[2] * J[3]);
        A[6] = J[3] * J[7] - J[4] * J[6];
        A[7] = -(J[0] * J[7] - J[1] * J[6]);
        A[8] = J[0] * J[4] - J[1] * J[3];
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
    static __device__ __forceinline__ void adj(const R* J, R* A) {  // J^-1 = A / det
        A[0] = J[3]; A[1] = -J[1];
        A[2] = -J[2]; A[3] = J[0];
    }
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
// Returns false when det C is small against the size of the terms it came from,
// det C <= 0.05 (1 + |X|)^3 (the FP32 det C and C^-1 then carry relative errors above about
// 1e-6): a near-singular or inverted deformation, whose point the caller recomputes in FP64.
template <typename R>
__device__ __forceinline__ bool neo_hooke_point(R mu, R lam, const R* H, R* out) {
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
    R nX = 0;
    #pragma unroll
    for (int t = 0; t < 9; ++t) nX += X[t] * X[t];
    const R sX = R(1) + sqrt(nX);
    const bool ok = detC > R(0.05) * sX * sX * sX;
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
    return ok;
}

// One quadrature point of a Neo-Hooke cell again in FP64 from the FP64 inputs (coordinates,
// reference tables, u): Jacobian, gradients, H = grad u, then neo_hooke_point; the outputs in
// FP32. For the rare points the FP32 form flags (kept out of line).
template <int K>
__device__ __forceinline__ void neo_point_fp64(const KernelArgs& a, const SubDev& sd, int cell, const uint16_t* cn,
                                            const int32_t* nodes, int q, float* out) {
    constexpr int NG = ElemT<K>::NG, NB = ElemT<K>::NB;
    double J[9], Ji[9], H[9], x0[3];
    const int n0 = nodes[cn[0]];
    for (int x = 0; x < 3; ++x) x0[x] = a.xd[(int64_t)n0 * 3 + x];
    for (int t = 0; t < 9; ++t) { J[t] = 0.0; H[t] = 0.0; }
    for (int k = 1; k < NG; ++k) {
        const int nk = nodes[cn[k]];
        for (int x = 0; x < 3; ++x) {
            const double o = a.xd[(int64_t)nk * 3 + x] - x0[x];
            for (int b = 0; b < 3; ++b) J[x * 3 + b] += o * sd.dM_d[(q * NG + k) * 3 + b];
        }
    }
    Mat<double, 3>::inv(J, Mat<double, 3>::det(J), Ji);
    for (int i = 0; i < NB; ++i) {
        double g[3] = {0.0, 0.0, 0.0};
        for (int b = 0; b < 3; ++b)
            for (int c = 0; c < 3; ++c) g[b] += sd.dN_d[(q * NB + i) * 3 + c] * Ji[c * 3 + b];
        const int64_t e3 = (int64_t)sd.ents[(int64_t)cell * NB + i] * 3;
        for (int c = 0; c < 3; ++c)
            for (int b = 0; b < 3; ++b) H[c * 3 + b] += a.phys.u_d[e3 + c] * g[b];
    }
    double o[NEO_POINT];
    neo_hooke_point<double>(a.phys.p0, a.phys.p1, H, o);
    for (int k = 0; k < NEO_POINT; ++k) out[k] = (float)o[k];
}

// ---------------------------------------------------------------------------------------
// per-CTA shared memory
// ---------------------------------------------------------------------------------------
constexpr int REC_RING = 3;     // records in flight: tile t (computing), t + G, t + 2G
constexpr int NODE_BYTES = 24;  // gathered coordinates per node (three 8-byte pieces)

// Shared-memory layout of a CTA, computed in one place for the kernel and the host.
struct SmemLayout {
    int shape, rec, coords, stage, chunk;  // chunk: cell tables, then the reduce's output buffer
};
__host__ __device__ inline int pad16i(int b) { return (b + 15) & ~15; }
__host__ __device__ inline int chunk_region_bytes(const KernelArgs& a) {
    const int out = pad16i(a.out_cap * 8);
    return a.chunk_bytes > out ? a.chunk_bytes : out;
}
__host__ __device__ inline SmemLayout smem_layout(const KernelArgs& a, int shape_bytes, int real_bytes) {
    SmemLayout L;
    int o = 0;
    L.shape = o; o += pad16i(shape_bytes);
    L.rec = o; o += REC_RING * pad16i(a.rec_cap);
    L.coords = o; o += 2 * a.node_cap * NODE_BYTES;
    L.stage = o; o += pad16i(a.stage_cap * real_bytes);
    L.chunk = o;
    return L;
}

// a physics constant in the kernel's precision: the host's FP32 copy, or the FP64 value
template <typename Real> __device__ __forceinline__ Real pconst(double d, float f);
template <> __device__ __forceinline__ float pconst<float>(double, float f) { return f; }
template <> __device__ __forceinline__ double pconst<double>(double d, float) { return d; }

template <typename Real> struct Pair;
template <> struct Pair<float> { using type = float2; };
template <> struct Pair<double> { using type = double2; };

// Packed multiply-add over a pair of quadrature points: one FFMA2 (sm_100+) for FP32.
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ double2 pfma(double2 a, double2 b, double2 c) {
    return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ double2 pmul(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
template <typename P> __device__ __forceinline__ P pzero();
template <> __device__ __forceinline__ float2 pzero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double2 pzero<double2>() { return make_double2(0.0, 0.0); }

// Reference tables in shared memory, one record per quadrature point q (element offsets):
//   dM[NG][DIM] at dm, dN[NB][DIM] at dn, N[NB] at n, w and sqrt(w) at w; every section starts on 16
//   bytes and the record stride qs is an odd multiple of 16 bytes, so the 8 lanes of a quarter
//   warp (lane = q) read their records with conflict-free 16-byte loads.
struct ShapeQ {
    int dm, dn, n, w, qs;
};
__host__ __device__ constexpr int round_up(int x, int m) { return (x + m - 1) / m * m; }
__host__ __device__ constexpr ShapeQ shape_q(int nb, int ng, int dim, int real_bytes) {
    const int v = 16 / real_bytes;
    ShapeQ s{};
    s.dm = 0;
    s.dn = round_up(ng * dim, v);
    s.n = s.dn + round_up(nb * dim, v);
    s.w = s.n + round_up(nb, v);
    int q = s.w + v;
    if ((q / v) % 2 == 0) q += v;
    s.qs = q;
    return s;
}

// Cell table layout (one per lane group), quadrature points taken in pairs (q0 = 2p,
// q1 = 2p+1; an odd count is padded with a zero-weight point):
//   grad[NQP][SP]    : at p*SP + i*6: (gx0, gx1, gy0, gy1, gz0, gz1), g = sqrt(detJ w) gradN
//   sq[NQP][2]       : detJ w per point (s squared)
//   cellp[4]         : per-cell material values
//   Neo-Hooke only:
//   bgrad[NQP][SP]   : B g per point and base function, laid out as grad (B = F^-T)
//   pairs[NQP][NEO_PAIR] : per point pair, T (6), c1, 2c2, s P (9), the two points interleaved
// SP (>= 6 NB) is chosen so that the lanes of a warp (lane = point, GS lanes per group, group
// tables GS words apart modulo 32) write their values to distinct shared-memory banks.
__host__ __device__ constexpr int table_sp(int nb, int nqp, int gs) {
    const int groups = gs >= 32 ? 1 : 32 / gs;
    const int pmax = nqp < gs / 2 ? nqp : gs / 2;
    for (int sp = nb * 6; sp < nb * 6 + 64; sp += 2) {
        unsigned mask = 0;
        bool ok = true;
        for (int g = 0; g < groups && ok; ++g)
            for (int p = 0; p < pmax && ok; ++p)
                for (int h = 0; h < 2 && ok; ++h) {
                    const int bank = (g * gs + p * sp + h) % 32;
                    if ((mask >> bank) & 1u) ok = false;
                    mask |= 1u << bank;
                }
        if (ok) return sp;
    }
    return nb * 6;
}
template <int K, int NQ, int PHYS, typename Real>
struct CellTable {
    static constexpr int NB = ElemT<K>::NB, GS = ElemT<K>::GS;
    static constexpr int NQP = (NQ + 1) / 2;
    static constexpr int SP = table_sp(NB, NQP, GS);
    static constexpr int GRAD = NQP * SP;
    static constexpr int SQ = NQP * 2;
    static constexpr int NEO = PHYS == PHYS_NEO ? NQP * SP + NQP * NEO_PAIR : 0;
    static constexpr int USED = GRAD + SQ + 4 + NEO;
    // group stride = GS (mod 32) elements
    static constexpr int REALS = USED + ((GS % 32 - USED % 32) + 32) % 32;
    static constexpr int BYTES = REALS * (int)sizeof(Real);
    static_assert(BYTES % 16 == 0, "group tables stay 16-byte aligned");
};

template <int K, int NQ, int PHYS, typename Real>
__host__ __device__ constexpr int cell_table_bytes() {
    return CellTable<K, NQ, PHYS, Real>::BYTES;
}

__host__ __device__ inline int pad16(int bytes) { return (bytes + 15) & ~15; }

// 16-byte vector loads of N (a multiple of 16 bytes) reals from a 16-byte aligned address
template <typename Real, int N>
__device__ __forceinline__ void lds16(const Real* p, Real* out) {
    if constexpr (sizeof(Real) == 4) {
        #pragma unroll
        for (int t = 0; t < N / 4; ++t) {
            const float4 v = ((const float4*)p)[t];
            out[4 * t] = v.x; out[4 * t + 1] = v.y; out[4 * t + 2] = v.z; out[4 * t + 3] = v.w;
        }
    } else {
        #pragma unroll
        for (int t = 0; t < N / 2; ++t) {
            const double2 v = ((const double2*)p)[t];
            out[2 * t] = v.x; out[2 * t + 1] = v.y;
        }
    }
}

// ---------------------------------------------------------------------------------------
// geometry of one cell by its lane group: lane q = quadrature point (NQ <= GS, NG <= GS).
// Node coordinates are loaded once per node (lane k loads node k) and shared with shuffles;
// the lane's reference-table record comes in 16-byte loads. Results go to the q-paired table
// layout; a padded point (odd NQ) is written as zeros.
// ---------------------------------------------------------------------------------------
constexpr int JT_STRIDE = 12;  // floats per point in a table of scaled inverse Jacobians (16-byte rows)

template <int K, int NQ, int PHYS, typename Real>
__device__ __forceinline__ void geometry_lanes(const KernelArgs& a, const SubDev& sd, const Real* shp, int cell,
                                               const uint16_t* cn, const char* xs, const int32_t* nodes, int lane,
                                               unsigned gmask, int gbase, Real* tb, int i0 = 0,
                                               int i1 = ElemT<K>::NB, bool lead = true, Real* jt = nullptr) {
    // [i0, i1): the base functions whose gradients this group writes (groups sharing a cell
    // split them); lead: the group that also writes the cell's point weights and factors;
    // jt: if given, each point's s J^-1 (row-major, JT_STRIDE apart) for callers that form the
    // gradients themselves
    using E = ElemT<K>;
    using CT = CellTable<K, NQ, PHYS, Real>;
    constexpr int NB = E::NB, NG = E::NG, DIM = E::DIM;
    constexpr ShapeQ SQL = shape_q(NB, NG, DIM, (int)sizeof(Real));
    constexpr int V = 16 / (int)sizeof(Real);
    static_assert(NQ <= E::GS && NG <= E::GS, "one lane per point and per node");
    Real* grad = tb;
    Real* sq = tb + CT::GRAD;
    Real* cellp = sq + CT::SQ;
    Real* neo = cellp + 4;
    // node offsets from node 0, shared through the group (coordinates: NODE_BYTES per node)
    Real off[NG][DIM];
    if constexpr (sizeof(Real) == 4) {
        const int ln = cn[lane < NG ? lane : 0];
        const float2 p0 = *(const float2*)(xs + ln * NODE_BYTES);
        const float2 p1 = *(const float2*)(xs + ln * NODE_BYTES + 8);
        const float2 p2 = *(const float2*)(xs + ln * NODE_BYTES + 16);
        const float h[3] = {p0.x, p0.y, p1.x}, l[3] = {p1.y, p2.x, p2.y};
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
        const double* x0 = (const double*)(xs + cn[0] * NODE_BYTES);
        #pragma unroll
        for (int k = 0; k < NG; ++k) {
            const double* xk = (const double*)(xs + cn[k] * NODE_BYTES);
            #pragma unroll
            for (int x = 0; x < DIM; ++x) off[k][x] = xk[x] - x0[x];
        }
    }
    if (lane >= NQ) return;
    const int q = lane;
    const Real* Q = shp + q * SQL.qs;
    Real J[DIM * DIM];
    {
        Real dm[round_up(NG * DIM, V)];
        lds16<Real, round_up(NG * DIM, V)>(Q + SQL.dm, dm);
        #pragma unroll
        for (int t = 0; t < DIM * DIM; ++t) J[t] = Real(0);
        #pragma unroll
        for (int k = 1; k < NG; ++k)
            #pragma unroll
            for (int x = 0; x < DIM; ++x)
                #pragma unroll
                for (int b = 0; b < DIM; ++b) J[x * DIM + b] += off[k][x] * dm[k * DIM + b];
    }
    Real dt = Mat<Real, DIM>::det(J);
    bool bad = !(dt > Real(0));
    // Ji = J^-1 scaled by s = sqrt(detJ w); every gradient below is then a plain product
    Real Ji[DIM * DIM];
    Real s;
    if constexpr (sizeof(Real) == 4) {
        // J^-1 s = adj(J) sqrt(w) / sqrt(detJ): one reciprocal square root, no division
        Real A[DIM * DIM];
        Mat<Real, DIM>::adj(J, A);
        float nJ = 0, nA = 0;
        #pragma unroll
        for (int t = 0; t < DIM * DIM; ++t) { nJ += J[t] * J[t]; nA += A[t] * A[t]; }
        // Frobenius condition estimate |J| |J^-1| = sqrt(nJ nA) / detJ against the threshold
        const float thr = a.phys.cond_threshold * (float)DIM;
        if (bad || nJ * nA > thr * thr * dt * dt) {
            double Jd[DIM * DIM], Jid[DIM * DIM];
            #pragma unroll
            for (int t = 0; t < DIM * DIM; ++t) Jd[t] = 0.0;
            const int n0 = nodes[cn[0]];
            double x0[DIM];
            #pragma unroll
            for (int x = 0; x < DIM; ++x) x0[x] = a.xd[(int64_t)n0 * a.dim + x];
            for (int k = 1; k < NG; ++k) {
                const int nk = nodes[cn[k]];
                for (int x = 0; x < DIM; ++x) {
                    const double o = a.xd[(int64_t)nk * a.dim + x] - x0[x];
                    for (int b = 0; b < DIM; ++b) Jd[x * DIM + b] += o * sd.dM_d[(q * NG + k) * DIM + b];
                }
            }
            const double dtd = Mat<double, DIM>::det(Jd);
            bad = !(dtd > 0.0);
            s = 0.f;
            if (!bad) {
                Mat<double, DIM>::inv(Jd, dtd, Jid);
                const double sd_ = sqrt(dtd * sd.w_d[q]);
                #pragma unroll
                for (int t = 0; t < DIM * DIM; ++t) Ji[t] = (float)(Jid[t] * sd_);
                s = (float)sd_;
            }
            dt = (float)dtd;
            if (q == 0 && lead) atomicAdd(&a.status->flagged, 1u);
        } else {
            const float r = rsqrtf(dt);
            const float sc = Q[SQL.w + 1] * r;  // sqrt(w) / sqrt(detJ)
            #pragma unroll
            for (int t = 0; t < DIM * DIM; ++t) Ji[t] = A[t] * sc;
            s = dt * sc;
        }
    } else {
        if (!bad) Mat<Real, DIM>::inv(J, dt, Ji);
        s = bad ? Real(0) : sqrt(dt * Q[SQL.w]);
        #pragma unroll
        for (int t = 0; t < DIM * DIM; ++t) Ji[t] *= s;
    }
    if (bad) {
        record_detj(a.status, sd.cellid[cell], (float)dt);
        s = Real(0);
        #pragma unroll
        for (int t = 0; t < DIM * DIM; ++t) Ji[t] = Real(0);
    }
    if (jt) {
        #pragma unroll
        for (int t = 0; t < DIM * DIM; ++t) jt[q * JT_STRIDE + t] = Ji[t];
    }
    // small elements keep the whole dN record in registers; large ones read it per node
    constexpr bool DN_REG = NB * DIM <= 32;
    Real dN[DN_REG ? round_up(NB * DIM, V) : 1];
    if constexpr (DN_REG) lds16<Real, round_up(NB * DIM, V)>(Q + SQL.dn, dN);
    const int p = q >> 1, hh = q & 1;
    const bool pad = (NQ & 1) && q == NQ - 1;
    if (lead) {
        sq[2 * p + hh] = s * s;
        if (pad) sq[2 * p + 1] = Real(0);
    }
    Real H[9];
    #pragma unroll
    for (int t = 0; t < 9; ++t) H[t] = Real(0);
    #pragma unroll
    for (int i = 0; i < NB; ++i) {
        if (i < i0 || i >= i1) continue;
        Real g[3] = {0, 0, 0};
        #pragma unroll
        for (int b = 0; b < DIM; ++b)
            #pragma unroll
            for (int c = 0; c < DIM; ++c) {
                if constexpr (DN_REG) g[b] += dN[i * DIM + c] * Ji[c * DIM + b];
                else g[b] += Q[SQL.dn + i * DIM + c] * Ji[c * DIM + b];
            }
        Real* o = grad + p * CT::SP + i * 6 + hh;
        o[0] = g[0];
        o[2] = g[1];
        o[4] = g[2];
        if (pad) { o[1] = Real(0); o[3] = Real(0); o[5] = Real(0); }
        if constexpr (PHYS == PHYS_NEO) {
            // H = grad u = sum_i u_i (x) gradN_i (function_gradient, common_values.jl:217-227),
            // accumulated with the scaled gradients and unscaled below
            const int64_t e3 = (int64_t)sd.ents[(int64_t)cell * NB + i] * 3;
            #pragma unroll
            for (int c = 0; c < 3; ++c) {
                Real uc;
                if constexpr (sizeof(Real) == 4) uc = a.phys.u_f[e3 + c];
                else uc = a.phys.u_d[e3 + c];
                #pragma unroll
                for (int J2 = 0; J2 < 3; ++J2) H[c * 3 + J2] += uc * g[J2];
            }
        }
    }
    if (q == 0 && lead) {
        Real scale = Real(1);
        if (a.phys.scale_f) {
            if constexpr (sizeof(Real) == 4) scale = a.phys.scale_f[sd.cellid[cell]];
            else scale = a.phys.scale_d[sd.cellid[cell]];
        }
        if constexpr (PHYS == PHYS_ELASTIC) {
            cellp[0] = pconst<Real>(a.phys.lam, a.phys.lam_f) * scale;
            cellp[1] = pconst<Real>(a.phys.mu, a.phys.mu_f) * scale;
        } else {
            cellp[0] = pconst<Real>(a.phys.p0, a.phys.p0_f) * scale;
            cellp[1] = pconst<Real>(a.phys.p1, a.phys.p1_f);
        }
    }
    if constexpr (PHYS == PHYS_NEO) {
        const Real is = s > Real(0) ? Real(1) / s : Real(0);
        #pragma unroll
        for (int t = 0; t < 9; ++t) H[t] *= is;
        Real nq[NEO_POINT];
        const bool ok = neo_hooke_point<Real>(pconst<Real>(a.phys.p0, a.phys.p0_f), pconst<Real>(a.phys.p1, a.phys.p1_f), H, nq);
        // the point's entries of the pair table (a padded partner point gets zeros) and B g_i
        // for the base functions this group writes (B = F^-T; the gradients written above are
        // read back by the same lane)
        auto write_point = [&](const Real* v) {
            if (lead) {
                Real* pp = neo + CT::GRAD + p * NEO_PAIR;
                constexpr int TK[6] = {0, 4, 8, 1, 2, 5};  // T00, T11, T22, T01, T02, T12
                #pragma unroll
                for (int k = 0; k < 6; ++k) pp[NEO_T + 2 * k + hh] = v[TK[k]];
                pp[NEO_C1 + hh] = v[18];
                pp[NEO_C2 + hh] = v[19];
                #pragma unroll
                for (int k = 0; k < 9; ++k) pp[NEO_SP + 2 * k + hh] = s * v[20 + k];
                if (pad) {
                    #pragma unroll
                    for (int k = 0; k < NEO_PAIR / 2; ++k) pp[2 * k + 1] = Real(0);
                }
            }
            #pragma unroll
            for (int i = 0; i < NB; ++i) {
                if (i < i0 || i >= i1) continue;
                const Real* gs = grad + p * CT::SP + i * 6 + hh;
                const Real gx = gs[0], gy = gs[2], gz = gs[4];
                Real* bd = neo + p * CT::SP + i * 6 + hh;
                #pragma unroll
                for (int x = 0; x < 3; ++x) bd[2 * x] = v[9 + 3 * x] * gx + v[9 + 3 * x + 1] * gy + v[9 + 3 * x + 2] * gz;
                if (pad) { bd[1] = Real(0); bd[3] = Real(0); bd[5] = Real(0); }
            }
        };
        write_point(nq);
        if constexpr (sizeof(Real) == 4) {
            // a near-singular or inverted deformation: this point again in FP64, its entries
            // rewritten (rare; last, so that little is live across the call)
            if (!ok && s > Real(0)) {
                float nd[NEO_POINT];
                neo_point_fp64<K>(a, sd, cell, cn, nodes, q, nd);
                write_point(nd);
                atomicAdd(&a.status->flagged, 1u);
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// phase B: the blocks of one cell into its owned columns; lane i = row base function
// ---------------------------------------------------------------------------------------
// One (item, row) block and the row's load entry into the tile's staging slots. The plan gives
// every (item, row) its own slot, so no two lanes write the same one; a block without a slot
// is a pattern miss unless it is exactly zero (assembler.jl:413-417, 459-467).
template <int NC_MAX, int nc, typename Real>
__device__ __forceinline__ void stage_block(const KernelArgs& a, const SubDev& sd, Real* stage, int f_off, int cell, int i, int j,
                                            int fslot, int slot, const Real* Kb, const Real* fe) {
    using P = typename Pair<Real>::type;
    constexpr int BSC = (nc * nc + 1) & ~1;
    if (a.do_k) {
        if (slot == SLOT_MISS) {
            #pragma unroll
            for (int x = 0; x < NC_MAX; ++x)
                #pragma unroll
                for (int y = 0; y < NC_MAX; ++y)
                    if (x < nc && y < nc && Kb[x * NC_MAX + y] != Real(0))
                        record_miss(a.status, sd.cellid[cell], i * nc + x, j * nc + y);
        } else {
            Real* dst = stage + slot * BSC;
            if (nc == 1) {
                dst[0] = Kb[0];
            } else {
                // column-major (b outer) so the reduce step reads in output order; an odd
                // count is padded with a zero so slots are pairs
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
        }
    }
    if (a.do_f && i == j) {
        Real* dst = stage + f_off + fslot * nc;
        #pragma unroll
        for (int x = 0; x < NC_MAX; ++x)
            if (x < nc) dst[x] = fe[x];
    }
}

template <int K, int NQ, int PHYS, typename Real, int EA = 0>
__device__ __forceinline__ void cell_blocks(const KernelArgs& a, const SubDev& sd, const char* R, const uint16_t* slot_rows,
                                            Real* stage, int f_off, const Real* tb, const Real* shp, int cell, int i, int it0,
                                            int it1, Real* ea_out = nullptr, const EaOut* eo = nullptr) {
    using E = ElemT<K>;
    using CT = CellTable<K, NQ, PHYS, Real>;
    using P = typename Pair<Real>::type;
    constexpr int NB = E::NB, NG = E::NG, DIM = E::DIM, NQP = CT::NQP;
    constexpr ShapeQ SQL = shape_q(NB, NG, DIM, (int)sizeof(Real));
    constexpr int NC_MAX = DIM;
    constexpr bool CACHE = NQP <= 4;  // keep the row function's table in registers
    // components per entity and staging stride, fixed by the physics (the host checks a.nc)
    constexpr int nc = PHYS == PHYS_HEAT ? 1 : DIM;
    const Real* grad = tb;
    const Real* sq = tb + CT::GRAD;
    const Real* cellp = sq + CT::SQ;
    const Real* neo = cellp + 4;
    const uint32_t* items = nullptr;
    if constexpr (EA == 0) items = (const uint32_t*)(R + ((const RecHead*)R)->off_items);
    P gi[CACHE ? NQP : 1][3];
    if constexpr (CACHE) {
        #pragma unroll
        for (int p = 0; p < NQP; ++p)
            #pragma unroll
            for (int c = 0; c < 3; ++c) gi[p][c] = *(const P*)(grad + p * CT::SP + i * 6 + 2 * c);
    }
    // volume load of this lane's function: sum_q N_i(q) detJ w (the body-force / source term)
    Real Fi = Real(0);
    if constexpr (PHYS != PHYS_NEO) {
        if (a.do_f) {
            #pragma unroll
            for (int q = 0; q < NQ; ++q) Fi += sq[q] * shp[q * SQL.qs + SQL.n + i];
        }
    }
    // EA 0: the block goes to the tile's staging slot; EA 1: to the cell's element matrix in
    // the two-phase scratch, [j][t][i] with t = y nc + x, then the load entries [x][i]; EA 2:
    // to the caller's element arrays (strides in eo)
    auto store_block = [&](int j, int fslot, int slot, const Real* Kb, const Real* fe) {
        if constexpr (EA == 2) {
            const int64_t cid = sd.cellid[cell];
            if (a.do_k) {
                Real* ko = (Real*)eo->ke + cid * eo->ks[0];
                #pragma unroll
                for (int y = 0; y < nc; ++y)
                    #pragma unroll
                    for (int x = 0; x < nc; ++x) ko[(i * nc + x) * eo->ks[1] + (j * nc + y) * eo->ks[2]] = Kb[x * NC_MAX + y];
            }
            if (a.do_f && i == j) {
                Real* fo = (Real*)eo->fe + cid * eo->fs[0];
                #pragma unroll
                for (int x = 0; x < nc; ++x) fo[(i * nc + x) * eo->fs[1]] = fe[x];
            }
        } else if constexpr (EA == 1) {
            constexpr int JS = ea_col_values(NB, nc);
            if (a.do_k) {
                #pragma unroll
                for (int y = 0; y < nc; ++y)
                    #pragma unroll
                    for (int x = 0; x < nc; ++x) ea_out[j * JS + (y * nc + x) * NB + i] = Kb[x * NC_MAX + y];
            }
            if (a.do_f && i == j) {
                #pragma unroll
                for (int x = 0; x < nc; ++x) ea_out[NB * JS + x * NB + i] = fe[x];
            }
        } else {
            stage_block<NC_MAX, nc, Real>(a, sd, stage, f_off, cell, i, j, fslot, slot, Kb, fe);
        }
    };
    if constexpr (PHYS == PHYS_HEAT || PHYS == PHYS_ELASTIC) {
        // M items at a time: their FFMA2 chains are independent, so one lane keeps more
        // instructions in flight
        auto items_m = [&](auto Mc, int it) {
            constexpr int M = decltype(Mc)::value;
            int jm[M], fsm[M], slm[M];
            #pragma unroll
            for (int m = 0; m < M; ++m) {
                if constexpr (EA != 0) {
                    jm[m] = it + m;  // every column of the cell
                    fsm[m] = slm[m] = 0;
                } else {
                    const uint32_t word = items[it + m];
                    jm[m] = (int)(word & 0xFF);
                    fsm[m] = (int)(word >> 16);
                    slm[m] = slot_rows[(it + m - it0) * NB + i];
                }
            }
            P G[M][DIM][DIM];
            #pragma unroll
            for (int m = 0; m < M; ++m)
                #pragma unroll
                for (int x = 0; x < DIM; ++x)
                    #pragma unroll
                    for (int y = 0; y < DIM; ++y) G[m][x][y] = pzero<P>();
            #pragma unroll
            for (int p = 0; p < NQP; ++p) {
                P ri[3], rj[M][3];
                #pragma unroll
                for (int c = 0; c < 3; ++c) {
                    if constexpr (CACHE) ri[c] = gi[p][c];
                    else ri[c] = *(const P*)(grad + p * CT::SP + i * 6 + 2 * c);
                    #pragma unroll
                    for (int m = 0; m < M; ++m) rj[m][c] = *(const P*)(grad + p * CT::SP + jm[m] * 6 + 2 * c);
                }
                #pragma unroll
                for (int m = 0; m < M; ++m) {
                    if constexpr (PHYS == PHYS_HEAT) {
                        #pragma unroll
                        for (int x = 0; x < DIM; ++x) G[m][0][0] = pfma(ri[x], rj[m][x], G[m][0][0]);
                    } else {
                        #pragma unroll
                        for (int x = 0; x < DIM; ++x)
                            #pragma unroll
                            for (int y = 0; y < DIM; ++y) G[m][x][y] = pfma(ri[x], rj[m][y], G[m][x][y]);
                    }
                }
            }
            #pragma unroll
            for (int m = 0; m < M; ++m) {
                Real Kb[NC_MAX * NC_MAX];
                Real fe[NC_MAX];
                if constexpr (PHYS == PHYS_HEAT) {
                    Kb[0] = cellp[0] * (G[m][0][0].x + G[m][0][0].y);
                    fe[0] = cellp[1] * Fi;
                } else {
                    Real g[DIM][DIM];
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x)
                        #pragma unroll
                        for (int y = 0; y < DIM; ++y) g[x][y] = G[m][x][y].x + G[m][x][y].y;
                    const Real lam = cellp[0], mu = cellp[1];
                    Real tr = 0;
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x) tr += g[x][x];
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x)
                        #pragma unroll
                        for (int y = 0; y < DIM; ++y) Kb[x * DIM + y] = lam * g[x][y] + mu * g[y][x] + (x == y ? mu * tr : Real(0));
                    #pragma unroll
                    for (int x = 0; x < DIM; ++x) fe[x] = Fi * pconst<Real>(a.phys.body[x], a.phys.body_f[x]);
                }
                store_block(jm[m], fsm[m], slm[m], Kb, fe);
            }
        };
        // one item at a time (two interleaved items measured slower: more instructions, same
        // registers)
        for (int it = it0; it < it1; ++it) items_m(std::integral_constant<int, 1>{}, it);
    } else {  // PHYS_NEO
        // K_ab(i, j) = sum_q delta_ab g_i.T g_j + c1 (B g_j)_a (B g_i)_b + 2c2 (B g_i)_a (B g_j)_b
        // (hyperelasticity.jl:254-276 with dP/dF from 157-176). The row lane keeps, per point
        // pair, its own B g_i and h_i = T g_i (T symmetric) and computes its residual entry
        // once; per item it reads the column's g_j and B g_j and runs the point pairs packed.
        const Real* bgt = neo;               // B g, laid out as grad
        const Real* pt = neo + CT::GRAD;     // per pair: T, c1, 2c2, s P
        P bgi[NQP][3], hi[NQP][3];
        P fr[3] = {pzero<P>(), pzero<P>(), pzero<P>()};
        #pragma unroll
        for (int p = 0; p < NQP; ++p) {
            const Real* pp = pt + p * NEO_PAIR;
            P g[3], T6[6], sP[9];
            #pragma unroll
            for (int c = 0; c < 3; ++c) {
                g[c] = *(const P*)(grad + p * CT::SP + i * 6 + 2 * c);
                bgi[p][c] = *(const P*)(bgt + p * CT::SP + i * 6 + 2 * c);
            }
            #pragma unroll
            for (int k = 0; k < 6; ++k) T6[k] = *(const P*)(pp + NEO_T + 2 * k);
            #pragma unroll
            for (int k = 0; k < 9; ++k) sP[k] = *(const P*)(pp + NEO_SP + 2 * k);
            // T rows from its distinct entries (T00, T11, T22, T01, T02, T12)
            const P Tr[3][3] = {{T6[0], T6[3], T6[4]}, {T6[3], T6[1], T6[5]}, {T6[4], T6[5], T6[2]}};
            #pragma unroll
            for (int x = 0; x < 3; ++x) {
                P h = pzero<P>(), r = fr[x];
                #pragma unroll
                for (int c = 0; c < 3; ++c) {
                    h = pfma(Tr[x][c], g[c], h);
                    r = pfma(sP[x * 3 + c], g[c], r);
                }
                hi[p][x] = h;
                fr[x] = r;
            }
        }
        // residual of the lane's own base function: sum_q s P g_i - s^2 N_i b
        Real fe_own[3];
        {
            Real nw = Real(0);
            #pragma unroll
            for (int q = 0; q < NQ; ++q) nw += sq[q] * shp[q * SQL.qs + SQL.n + i];
            #pragma unroll
            for (int x = 0; x < 3; ++x) fe_own[x] = (fr[x].x + fr[x].y) - nw * pconst<Real>(a.phys.body[x], a.phys.body_f[x]);
        }
        for (int it = it0; it < it1; ++it) {
            int j = it, fslot = 0, slot = 0;
            if constexpr (EA == 0) {
                const uint32_t word = items[it];
                j = (int)(word & 0xFF);
                fslot = (int)(word >> 16);
                slot = slot_rows[(it - it0) * NB + i];
            }
            P K[3][3], t = pzero<P>();
            #pragma unroll
            for (int x = 0; x < 3; ++x)
                #pragma unroll
                for (int y = 0; y < 3; ++y) K[x][y] = pzero<P>();
            #pragma unroll
            for (int p = 0; p < NQP; ++p) {
                const Real* pp = pt + p * NEO_PAIR;
                const P c1 = *(const P*)(pp + NEO_C1), c2 = *(const P*)(pp + NEO_C2);
                P gj[3], c1b[3], c2b[3];
                #pragma unroll
                for (int c = 0; c < 3; ++c) {
                    gj[c] = *(const P*)(grad + p * CT::SP + j * 6 + 2 * c);
                    const P b = *(const P*)(bgt + p * CT::SP + j * 6 + 2 * c);
                    c1b[c] = pmul(c1, b);
                    c2b[c] = pmul(c2, b);
                }
                #pragma unroll
                for (int c = 0; c < 3; ++c) t = pfma(hi[p][c], gj[c], t);
                #pragma unroll
                for (int x = 0; x < 3; ++x)
                    #pragma unroll
                    for (int y = 0; y < 3; ++y) K[x][y] = pfma(bgi[p][x], c2b[y], pfma(c1b[x], bgi[p][y], K[x][y]));
            }
            Real Kb[NC_MAX * NC_MAX];
            const Real tij = t.x + t.y;
            #pragma unroll
            for (int x = 0; x < 3; ++x)
                #pragma unroll
                for (int y = 0; y < 3; ++y) Kb[x * 3 + y] = (K[x][y].x + K[x][y].y) + (x == y ? tij : Real(0));
            store_block(j, fslot, slot, Kb, fe_own);
        }
    }
}

// ---------------------------------------------------------------------------------------
// two-phase form, phase B: the items' blocks come from the cell's element matrix in global
// memory (written by element_kernel); lane i = row base function, coalesced over i. The
// scratch keeps a column's values in the staging slot's own order (t = y nc + x), so each value
// is copied global -> shared with cp.async: every lane issues all its copies without waiting,
// and the tile waits for them once, before the reduce (rows without a pattern entry are loaded
// into registers instead and checked for non-zeros).
// ---------------------------------------------------------------------------------------
template <typename Real>
__device__ __forceinline__ void async_copy(Real* dst, const Real* src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(Real) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}

template <int K, int PHYS, typename Real>
__device__ __forceinline__ void gather_blocks(const KernelArgs& a, const SubDev& sd, const char* R, const uint16_t* slot_rows,
                                              Real* stage, int f_off, const Real* __restrict__ ea, int cell, int i, int it0,
                                              int it1) {
    using E = ElemT<K>;
    constexpr int NB = E::NB, NC_MAX = E::DIM;
    constexpr int nc = PHYS == PHYS_HEAT ? 1 : E::DIM;
    constexpr int JS = ea_col_values(NB, nc);
    constexpr int BSC = (nc * nc + 1) & ~1;
    const uint32_t* items = (const uint32_t*)(R + ((const RecHead*)R)->off_items);
    for (int it = it0; it < it1; ++it) {
        const uint32_t word = items[it];
        const int j = (int)(word & 0xFF);
        const int slot = slot_rows[(it - it0) * NB + i];
        if (a.do_k) {
            if (slot != SLOT_MISS) {
                Real* dst = stage + slot * BSC;
                #pragma unroll
                for (int t = 0; t < nc * nc; ++t) async_copy(dst + t, ea + j * JS + t * NB + i);
            } else {
                // no pattern entry: allowed only for exact zeros (assembler.jl:413-417, 459-467)
                #pragma unroll
                for (int y = 0; y < nc; ++y)
                    #pragma unroll
                    for (int x = 0; x < nc; ++x)
                        if (__ldcs(ea + j * JS + (y * nc + x) * NB + i) != Real(0))
                            record_miss(a.status, sd.cellid[cell], i * nc + x, j * nc + y);
            }
        }
        if (a.do_f && i == j) {
            Real* dst = stage + f_off + (int)(word >> 16) * nc;
            #pragma unroll
            for (int x = 0; x < nc; ++x) async_copy(dst + x, ea + NB * JS + x * NB + i);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// ---------------------------------------------------------------------------------------
// the cells of one subdomain in a tile
// ---------------------------------------------------------------------------------------
template <int K, int NQ, int PHYS, typename Real, bool EAK = false>
__device__ __forceinline__ void process_segment(const KernelArgs& a, const SubDev& sd, const Real* shp, const RecSeg& g,
                                                const char* R, const char* xs, Real* stage, char* chunk) {
    using E = ElemT<K>;
    using CT = CellTable<K, NQ, PHYS, Real>;
    constexpr int NB = E::NB, NG = E::NG, DIM = E::DIM, GS = E::GS;
    const RecHead* H = (const RecHead*)R;
    const int32_t* cells = (const int32_t*)(R + H->off_cells);
    const int32_t* nodes = (const int32_t*)(R + H->off_nodes);
    const uint16_t* conn = (const uint16_t*)(R + g.conn_off);
    const uint16_t* slots = (const uint16_t*)(R + g.slot_off);
    const int f_off = H->n_slots * a.bs;
    const int tid = threadIdx.x;
    // one lane group per cell (round robin), each with a private table buffer: the group
    // computes its cell's geometry (lane = quadrature point), syncs within the warp, then
    // its lanes (= row base functions) compute and stage the blocks
    const int ngrp = a.groups[g.sub];  // <= THREADS / GS, bounded by the table memory
    const int lane = tid % GS, grp = tid / GS;
    const unsigned gmask = GS >= 32 ? 0xFFFFFFFFu : (((1u << GS) - 1u) << ((tid & 31) / GS * GS));
    Real* tb = (Real*)(chunk + grp * CT::BYTES);
    const uint16_t* gt = (const uint16_t*)(R + g.gt_off);
    const RecTask* tasks = (const RecTask*)(R + H->off_tasks);
    const Real* ea = (const Real*)a.ea[g.sub];
    if (EAK || ea) {
        // two-phase form: no geometry here, the blocks are loaded
        const int64_t es = a.ea_stride[g.sub];
        for (int pg = grp; grp < ngrp && pg < g.n_grp; pg += ngrp) {
            const int t1 = gt[pg + 1];
            for (int ti = gt[pg]; ti < t1; ++ti) {
                const RecTask tk = tasks[ti];
                const int cell = cells[tk.cell];
                if (lane < NB)
                    gather_blocks<K, PHYS, Real>(a, sd, R, slots + (tk.item_begin - g.item_begin) * NB, stage, f_off,
                                                 ea + (int64_t)cell * es, cell, lane, tk.item_begin, tk.item_end);
            }
        }
        return;
    }
    if constexpr (!EAK) {
    // the plan's groups run on this CTA's groups round robin (the same when the counts agree)
    for (int pg = grp; grp < ngrp && pg < g.n_grp; pg += ngrp) {
        const int t1 = gt[pg + 1];
        for (int ti = gt[pg]; ti < t1; ++ti) {
            const RecTask tk = tasks[ti];
            const int cell = cells[tk.cell];
            geometry_lanes<K, NQ, PHYS, Real>(a, sd, shp, cell, conn + (tk.cell - g.cell_begin) * NG, xs, nodes, lane, gmask,
                                              (tid & 31) - lane, tb);
            __syncwarp(gmask);
            if (lane < NB)
                cell_blocks<K, NQ, PHYS, Real>(a, sd, R, slots + (tk.item_begin - g.item_begin) * NB, stage, f_off, tb, shp, cell,
                                               lane, tk.item_begin, tk.item_end);
            __syncwarp(gmask);  // the next task overwrites the table
        }
    }
    }
}

// ---------------------------------------------------------------------------------------
// reduce: one lane per owned (entity n, row entity r) block. The block's contributions sit
// in consecutive slots in cell order; they are summed compensated, rounded to FP64 and
// stored: nc columns of nc rows.
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

// TMA bulk stores shared -> global (both addresses 16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_store(double* dst, uint32_t src, int bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// One f entry (owned entity e, component x): its cells' contributions in cell order.
template <int NC, typename Real>
__device__ __forceinline__ void f_entry(const KernelArgs& a, const char* R, const Real* stage, int idx) {
    const RecHead* H = (const RecHead*)R;
    const int32_t* eid = (const int32_t*)(R + H->off_eid);
    const uint32_t* fk = (const uint32_t*)(R + H->off_fk);
    const int e = idx / NC, x = idx - e * NC;
    const uint32_t w = fk[e];
    const int fb = (int)(w & 0xFFFF), kcnt = (int)(w >> 16);
    const int64_t gi = (int64_t)eid[e] * NC + x;
    const Real* v = stage + H->n_slots * ((NC * NC + 1) & ~1) + fb * NC + x;
    double out;
    if constexpr (sizeof(Real) == 4) {
        if (a.compensated) {
            float2 acc = make_float2(0.f, 0.f);
            if (!a.fillzero) acc_set(acc, a.f[gi]);
            for (int k = 0; k < kcnt; ++k) acc_add(acc, v[k * NC]);
            out = acc_value(acc);
        } else {
            float acc = 0.f;
            for (int k = 0; k < kcnt; ++k) acc += v[k * NC];
            out = float_to_double(acc);
            if (!a.fillzero) out += a.f[gi];
        }
    } else {
        double acc = a.fillzero ? 0.0 : a.f[gi];
        for (int k = 0; k < kcnt; ++k) acc += v[k * NC];
        out = acc;
    }
    __stcs(a.f + gi, out);
}

// Per pass: blocks in the plan's order (most contributions first, so the lanes of a warp run
// loops of equal length and read consecutive slots; the lane does not change any value) are
// summed into the shared output buffer in nzval order; then each contiguous nzval range is
// written by one bulk store (its 16-byte aligned middle) and plain stores (its ends). With an
// nzval pointer that is only 8-byte aligned, all threads copy the buffer out instead. The f
// entries ride on the lanes of the last pass that have no block left.
template <int NC, typename Real>
__device__ __forceinline__ void reduce_tile(const KernelArgs& a, const char* R, const Real* stage, double* outb) {
    constexpr int NCC = NC * NC, BS = (NCC + 1) & ~1, NP = BS / 2;
    const RecHead* H = (const RecHead*)R;
    const int nf = a.do_f ? H->n_ent * NC : 0;
    if (!a.do_k) {
        for (int idx = threadIdx.x; idx < nf; idx += THREADS) f_entry<NC, Real>(a, R, stage, idx);
        return;
    }
    const RecEnt* ents = (const RecEnt*)(R + H->off_ent);
    const uint32_t* red = (const uint32_t*)(R + H->off_red);
    const RecRun* runs = (const RecRun*)(R + H->off_runs);
    const RecPass* passes = (const RecPass*)(R + H->off_pass);
    const RecRng* rngs = (const RecRng*)(R + H->off_rng);
    // TMA bulk stores into device memory; plain stores into host memory or unaligned nzval
    const bool bulk = !a.host_out && ((uintptr_t)a.nzval & 15) == 0;
    const uint32_t outb_s = (uint32_t)__cvta_generic_to_shared(outb);
    const int n_pass = H->n_pass;
    for (int p = 0; p < n_pass; ++p) {
        const RecPass P = passes[p];
        if (p > 0) {  // the previous pass's copies still read the buffer
            bulk_wait_read();
            __syncthreads();
        }
        const int end = P.red_end + (p + 1 == n_pass ? nf : 0);
        int u = P.run_begin;  // run of the current block (positions only grow)
        // snake order: round k takes positions k THREADS + (k odd ? THREADS - 1 - tid : tid), so
        // a thread's second block (fewer contributions, the order being by count) is the lighter
        // the heavier its first one was
        for (int k = 0;; ++k) {
            const int pos = P.red_begin + k * THREADS + ((k & 1) ? THREADS - 1 - (int)threadIdx.x : (int)threadIdx.x);
            if (pos >= end) break;
            if (pos >= P.red_end) {
                f_entry<NC, Real>(a, R, stage, pos - P.red_end);
                continue;
            }
            const uint32_t key = red[pos];
            const int e = (int)(key >> RED_RANK_BITS), r = (int)(key & ((1u << RED_RANK_BITS) - 1));
            while (u + 1 < P.run_end && runs[u + 1].first <= pos) ++u;
            const int4 ru = *(const int4*)(runs + u);  // first, count, base, nblk
            const int s0 = ru.z + (pos - ru.x), ds = ru.w, cnt = ru.y;
            const RecEnt en = ents[e];
            const int64_t L = en.L;
            double out[NCC];
            if constexpr (sizeof(Real) == 4) {
                if (a.compensated) {
                    float2 hi[NP], lo[NP];
                    #pragma unroll
                    for (int t = 0; t < NP; ++t) { hi[t] = make_float2(0.f, 0.f); lo[t] = make_float2(0.f, 0.f); }
                    int k = 0;
                    if (!a.fillzero) {
                        const int64_t c0 = en.colbase + (int64_t)NC * r;
                        float hv[BS], lv[BS];
                        #pragma unroll
                        for (int t = 0; t < BS; ++t) { hv[t] = 0.f; lv[t] = 0.f; }
                        #pragma unroll
                        for (int b = 0; b < NC; ++b)
                            #pragma unroll
                            for (int x = 0; x < NC; ++x) {
                                float2 q;
                                acc_set(q, a.nzval[c0 + b * L + x]);
                                hv[b * NC + x] = q.x;
                                lv[b * NC + x] = q.y;
                            }
                        #pragma unroll
                        for (int t = 0; t < NP; ++t) { hi[t] = make_float2(hv[2 * t], hv[2 * t + 1]); lo[t] = make_float2(lv[2 * t], lv[2 * t + 1]); }
                    } else if (cnt > 0) {
                        const float2* v = (const float2*)(stage + s0 * BS);
                        #pragma unroll
                        for (int t = 0; t < NP; ++t) hi[t] = v[t];
                        k = 1;
                        if (cnt == 2) {
                            // two contributions: the pair (a, b) itself is rounded below, the
                            // same double as the TwoSum pair of a + b
                            const float2* w = (const float2*)(stage + (s0 + ds) * BS);
                            #pragma unroll
                            for (int t = 0; t < NP; ++t) lo[t] = w[t];
                            k = 2;
                        }
                    }
                    for (; k < cnt; ++k) {
                        const float2* v = (const float2*)(stage + (s0 + k * ds) * BS);
                        #pragma unroll
                        for (int t = 0; t < NP; ++t) acc_add2(hi[t], lo[t], v[t]);
                    }
                    if (a.fillzero && cnt <= 1) {
                        // a single contribution is its own exact sum: no low word to round in
                        // (blocks of equal counts are adjacent, so warps take one branch)
                        #pragma unroll
                        for (int t = 0; t < NP; ++t) {
                            out[2 * t] = float_to_double(hi[t].x);
                            if (2 * t + 1 < NCC) out[2 * t + 1] = float_to_double(hi[t].y);
                        }
                    } else {
                        // branch-free rounding of every entry; the block's few entries whose sum
                        // needs care (zero, tiny, a power of two) are redone exactly
                        bool rare = false;
                        #pragma unroll
                        for (int t = 0; t < NCC / 2; ++t) pair2_to_double(hi[t], lo[t], out[2 * t], out[2 * t + 1], rare);
                        if constexpr (NCC & 1) out[NCC - 1] = pair1_to_double(hi[NP - 1].x, lo[NP - 1].x, rare);
                        if (rare) {
                            #pragma unroll
                            for (int t = 0; t < NP; ++t) {
                                out[2 * t] = pair_to_double(hi[t].x, lo[t].x);
                                if (2 * t + 1 < NCC) out[2 * t + 1] = pair_to_double(hi[t].y, lo[t].y);
                            }
                        }
                    }
                } else {
                    // packed FP32 sums in cell order, each rounded exactly to FP64
                    float2 acc[NP];
                    #pragma unroll
                    for (int t = 0; t < NP; ++t) acc[t] = make_float2(0.f, 0.f);
                    #pragma unroll 4
                    for (int k = 0; k < cnt; ++k) {
                        const float2* v = (const float2*)(stage + (s0 + k * ds) * BS);
                        #pragma unroll
                        for (int t = 0; t < NP; ++t) acc[t] = __fadd2_rn(acc[t], v[t]);
                    }
                    #pragma unroll
                    for (int t = 0; t < NP; ++t) {
                        out[2 * t] = float_to_double(acc[t].x);
                        if (2 * t + 1 < NCC) out[2 * t + 1] = float_to_double(acc[t].y);
                    }
                    if (!a.fillzero) {
                        const int64_t c0 = en.colbase + (int64_t)NC * r;
                        #pragma unroll
                        for (int b = 0; b < NC; ++b)
                            #pragma unroll
                            for (int x = 0; x < NC; ++x) out[b * NC + x] += a.nzval[c0 + b * L + x];
                    }
                }
            } else {
                double acc[NCC];
                #pragma unroll
                for (int t = 0; t < NCC; ++t) acc[t] = 0.0;
                if (!a.fillzero) {
                    const int64_t c0 = en.colbase + (int64_t)NC * r;
                    #pragma unroll
                    for (int b = 0; b < NC; ++b)
                        #pragma unroll
                        for (int x = 0; x < NC; ++x) acc[b * NC + x] = a.nzval[c0 + b * L + x];
                }
                for (int k = 0; k < cnt; ++k) {
                    const Real* v = stage + (s0 + k * ds) * BS;
                    #pragma unroll
                    for (int t = 0; t < NCC; ++t) acc[t] += v[t];
                }
                #pragma unroll
                for (int t = 0; t < NCC; ++t) out[t] = acc[t];
            }
            double* o = outb + en.out_off + NC * r;
            #pragma unroll
            for (int b = 0; b < NC; ++b)
                #pragma unroll
                for (int x = 0; x < NC; ++x) o[b * L + x] = out[b * NC + x];
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // buffer writes -> bulk copies
        __syncthreads();
        if (bulk) {
            // one thread per range (the last threads of the CTA, which hold the fewest blocks):
            // the ends with plain stores, the aligned middle with one bulk store of its own group
            const int nrg = P.rng_end - P.rng_begin;
            for (int q = THREADS - 1 - (int)threadIdx.x; q < nrg; q += THREADS) {
                const RecRng g = rngs[P.rng_begin + q];
                const int64_t e = g.nz0 + g.len;
                if (g.nz0 & 1) __stcs(a.nzval + g.nz0, outb[g.buf_off]);
                if (e & 1) __stcs(a.nzval + e - 1, outb[g.buf_off + g.len - 1]);  // never the head element
                const int64_t a0 = g.nz0 + (g.nz0 & 1), a1 = e & ~(int64_t)1;
                if (a1 > a0) bulk_store(a.nzval + a0, outb_s + (uint32_t)(g.buf_off + (a0 - g.nz0)) * 8u, (int)(a1 - a0) * 8);
                bulk_commit();
            }
        } else {
            // host memory (pinned, through its mapping) or an nzval that is only 8-byte aligned:
            // one warp per range, so every warp has stores in flight; 16-byte stores for the
            // aligned pairs when nzval is 16-byte aligned (the buffer keeps each range's parity)
            const int warp = (int)threadIdx.x >> 5, ln = (int)threadIdx.x & 31;
            const bool v2 = ((uintptr_t)a.nzval & 15) == 0;
            for (int gi = P.rng_begin + warp; gi < P.rng_end; gi += THREADS / 32) {
                const RecRng g = rngs[gi];
                if (v2) {
                    const int64_t e = g.nz0 + g.len;
                    const int64_t a0 = g.nz0 + (g.nz0 & 1), a1 = e & ~(int64_t)1;
                    if (ln == 0 && (g.nz0 & 1)) __stcs(a.nzval + g.nz0, outb[g.buf_off]);
                    if (ln == 1 && (e & 1)) __stcs(a.nzval + e - 1, outb[g.buf_off + g.len - 1]);  // never the head element
                    const double2* src = (const double2*)(outb + g.buf_off + (a0 - g.nz0));
                    double2* dst = (double2*)(a.nzval + a0);
                    for (int64_t k = ln; 2 * k < a1 - a0; k += 32) __stcs(dst + k, src[k]);
                } else {
                    for (int k = ln; k < g.len; k += 32) __stcs(a.nzval + g.nz0 + k, outb[g.buf_off + k]);
                }
            }
            if (p + 1 < n_pass) __syncthreads();
        }
    }
    // the next tile writes its cell tables over the buffer: each issuing thread waits until its
    // bulk stores have read it (the CTA barrier of the next tile orders the rest)
    bulk_wait_read();
}

// ---------------------------------------------------------------------------------------
// asynchronous copies
// ---------------------------------------------------------------------------------------
constexpr long long WAIT_LIMIT = 1ll << 24;  // mbarrier polls before a copy counts as lost

// bounded wait on an mbarrier phase (TMA bulk copy completion)
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

// one TMA bulk copy global -> shared, completing on an mbarrier (bytes: multiple of 16,
// both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, int bytes, uint32_t bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst), "l"(src),
                 "r"(bytes), "r"(bar)
                 : "memory");
}

// gather the coordinates of a tile's nodes (three 8-byte pieces per node) into shared memory
template <typename Real>
__device__ __forceinline__ void gather_nodes(const KernelArgs& a, const char* R, char* xs) {
    const RecHead* H = (const RecHead*)R;
    const int32_t* nodes = (const int32_t*)(R + H->off_nodes);
    const char* src = sizeof(Real) == 4 ? (const char*)a.xf6 : (const char*)a.xd3;
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(xs);
    const int n = 3 * H->n_nodes;
    for (int k = threadIdx.x; k < n; k += THREADS) {
        const int nd = k / 3, piece = k - nd * 3;
        const char* p = src + (int64_t)nodes[nd] * NODE_BYTES + piece * 8;
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst + k * 8), "l"(p) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// ---------------------------------------------------------------------------------------
// the kernel: persistent CTAs, tiles blockIdx.x + it * gridDim.x
// ---------------------------------------------------------------------------------------
// EAK: the gather-only form for subdomains whose element matrices all come precomputed (no
// geometry code, no coordinates; fewer registers, so three CTAs share an SM)
template <int K0, int Q0, int K1, int Q1, int K2, int Q2, int PHYS, typename Real, bool EAK = false>
__global__ void __launch_bounds__(THREADS, EAK ? 3 : 2) tile_kernel(const KernelArgs a, const Real* __restrict__ shape_g, int shape_bytes,
                                                           int shape_off1, int shape_off2) {
    extern __shared__ __align__(128) char smem_raw[];
    __shared__ __align__(8) unsigned long long bars[1 + REC_RING];  // shape tables, record ring
    const SmemLayout lay = smem_layout(a, shape_bytes, (int)sizeof(Real));
    {
        // the host sized the allocation from the same layout; refuse to run past it
        uint32_t dyn;
        asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
        if ((uint32_t)(lay.chunk + chunk_region_bytes(a)) > dyn) {
            if (threadIdx.x == 0) atomicAdd(&a.status->timeout, 1u);
            return;
        }
    }
    Real* shape = (Real*)(smem_raw + lay.shape);
    char* rec_ring = smem_raw + lay.rec;
    char* xs_ring = smem_raw + lay.coords;
    Real* stage = (Real*)(smem_raw + lay.stage);
    char* chunk = smem_raw + lay.chunk;
    const int rec_stride = pad16i(a.rec_cap), xs_stride = a.node_cap * NODE_BYTES;
    const int tid = threadIdx.x;
    const int G = gridDim.x;
    const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(&bars[0]);
    auto rec_bar = [&](int b) { return bar0 + 8u * (uint32_t)(1 + b); };
    auto issue_record = [&](int64_t o, int64_t o1, int b) {
        bulk_load((uint32_t)__cvta_generic_to_shared(rec_ring + b * rec_stride), a.rec + o, (int)(o1 - o), rec_bar(b));
    };
    int64_t pf0 = 0, pf1 = 0;  // thread 0: offsets of the record it issues next (loaded a tile ahead)
    int t = blockIdx.x;
    if (tid == 0) {
        for (int b = 0; b < 1 + REC_RING; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8u * b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // no shape tables when every subdomain's element matrices come precomputed
        if (shape_bytes > 0) bulk_load((uint32_t)__cvta_generic_to_shared(shape), shape_g, shape_bytes, bar0);
        else asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar0) : "memory");
        if (t < a.n_tiles) issue_record(a.rec_off[t], a.rec_off[t + 1], 0);
        if (t + G < a.n_tiles) issue_record(a.rec_off[t + G], a.rec_off[t + G + 1], 1);
        if (t + 2 * G < a.n_tiles) { pf0 = a.rec_off[t + 2 * G]; pf1 = a.rec_off[t + 2 * G + 1]; }
    }
    __syncthreads();  // the initialised barriers are visible to every thread
    // node coordinates are needed unless every subdomain's element matrices come precomputed
    bool geo = false;
    if constexpr (!EAK)
        for (int s = 0; s < a.n_sub; ++s) geo |= a.ea[s] == nullptr;
    bool failed = false;
    if (t < a.n_tiles) {
        if (!mbar_wait(rec_bar(0), 0, WAIT_LIMIT)) failed = true;
        else if (geo) gather_nodes<Real>(a, rec_ring, xs_ring);
    }
    if (!failed && !mbar_wait(bar0, 0, WAIT_LIMIT)) failed = true;
    int it = 0;
    // The gather-only form needs no barrier at the top of a tile after the first: its staging
    // slots and output buffer are separate, the reduce's barrier before the bulk stores follows
    // its last read of the slots, and a record that did not arrive is caught at the barrier
    // after the copies. Warps that finish a tile early start the next tile's copies.
    for (; t < a.n_tiles; ++it, t += G) {
        if (!EAK || it == 0) {
            asm volatile("cp.async.wait_all;" ::: "memory");
            if (__syncthreads_or(failed)) break;  // this tile's record and coordinates are in place
        }
        const char* R = rec_ring + (it % REC_RING) * rec_stride;
        const char* xs = xs_ring + (it & 1) * xs_stride;
        // keep the pipeline full: record of t + 2G (the gather-only form issues it after the
        // copies, once every thread is past the previous tile), coordinates of t + G
        if (!EAK && tid == 0 && t + 2 * G < a.n_tiles) {
            issue_record(pf0, pf1, (it + 2) % REC_RING);
            if (t + 3 * G < a.n_tiles) { pf0 = a.rec_off[t + 3 * G]; pf1 = a.rec_off[t + 3 * G + 1]; }
        }
        if (t + G < a.n_tiles) {
            const int nb = (it + 1) % REC_RING;
            if (!mbar_wait(rec_bar(nb), (uint32_t)(((it + 1) / REC_RING) & 1), WAIT_LIMIT))
                failed = true;
            else if (geo)
                gather_nodes<Real>(a, rec_ring + nb * rec_stride, xs_ring + ((it + 1) & 1) * xs_stride);

        }
        const RecHead* H = (const RecHead*)R;
        const int n_seg = H->n_seg;
        for (int gi = 0; gi < n_seg; ++gi) {
            if (!EAK && gi) __syncthreads();  // table buffers are laid out per element kind (none in the gather-only form)
            const RecSeg g = ((const RecSeg*)(R + sizeof(RecHead)))[gi];
            static_assert(sizeof(RecSeg) % 16 == 0, "segment entries are 16-byte multiples");
            if (g.sub == 0) {
                process_segment<K0, Q0, PHYS, Real, EAK>(a, a.sub[0], shape, g, R, xs, stage, chunk);
            } else if constexpr (K1 >= 0) {
                if (g.sub == 1) {
                    process_segment<K1, Q1, PHYS, Real, EAK>(a, a.sub[1], (const Real*)((const char*)shape + shape_off1), g, R, xs,
                                                        stage, chunk);
                } else if constexpr (K2 >= 0) {
                    process_segment<K2, Q2, PHYS, Real, EAK>(a, a.sub[2], (const Real*)((const char*)shape + shape_off2), g, R, xs,
                                                        stage, chunk);
                }
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");  // this thread's slot copies (two-phase form)
        if constexpr (EAK) {
            if (__syncthreads_or(failed)) break;  // all staging slots written; the next record arrived
            if (tid == 0 && t + 2 * G < a.n_tiles) {
                issue_record(pf0, pf1, (it + 2) % REC_RING);
                if (t + 3 * G < a.n_tiles) { pf0 = a.rec_off[t + 3 * G]; pf1 = a.rec_off[t + 3 * G + 1]; }
            }
        } else {
            __syncthreads();  // all staging slots written
        }
        if (a.nc == 3) reduce_tile<3, Real>(a, R, stage, (double*)chunk);
        else if (a.nc == 2) reduce_tile<2, Real>(a, R, stage, (double*)chunk);
        else reduce_tile<1, Real>(a, R, stage, (double*)chunk);
        if constexpr (EAK)
            if (!a.do_k) __syncthreads();  // the f entries have read the staging slots
    }
    bulk_wait_all();  // this CTA's output stores have completed
    if (t < a.n_tiles) {
        // a copy was lost: report it, and wait (bounded) for this CTA's copies still in
        // flight before its shared memory is released
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (tid == 0) {
            atomicAdd(&a.status->timeout, 1u);
            mbar_wait(bar0, 0, WAIT_LIMIT);
            for (int d = 0; d < 2; ++d) {
                const int tt = t + d * G;
                if (tt < a.n_tiles) mbar_wait(rec_bar((it + d) % REC_RING), (uint32_t)(((it + d) / REC_RING) & 1), WAIT_LIMIT);
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// element matrices: one lane group per cell computes the geometry (lane = quadrature point),
// then every column j of Ke and the load vector (lane = row function i) into out + cell *
// stride, laid out [j][t][i] (t = y nc + x, the block's entries column by column) and then
// fe [x][i]. Phase A of the two-phase assembly; the element-assembly output of the GPU how-to
// (gpu_assembly.jl:265-303) in this layout.
// ---------------------------------------------------------------------------------------
template <int K, int NQ, int PHYS, typename Real>
struct EaGroup {
    static constexpr int NG = ElemT<K>::NG;
    static constexpr int TB = CellTable<K, NQ, PHYS, Real>::BYTES;  // cell table
    static constexpr int XS = (NG * NODE_BYTES + 15) / 16 * 16;     // node coordinates
    static constexpr int ND = (NG * 4 + 15) / 16 * 16;              // node ids
    static constexpr int CN = (NG * 2 + 15) / 16 * 16;              // local node numbers
    static constexpr int BYTES = TB + XS + ND + CN;
};

template <int K, int NQ, int PHYS, typename Real>
__host__ __device__ constexpr int element_smem_bytes(int shape_bytes) {
    return pad16(shape_bytes) + (THREADS / ElemT<K>::GS) * EaGroup<K, NQ, PHYS, Real>::BYTES;
}

// MODE 1: into the two-phase scratch; MODE 2: into the caller's arrays (EaOut strides)
template <int K, int NQ, int PHYS, typename Real, int MODE>
__global__ void __launch_bounds__(THREADS, 2) element_kernel(const KernelArgs a, const SubDev sd, const Real* __restrict__ shape_g,
                                                              int shape_bytes, const EaOut eo) {
    using E = ElemT<K>;
    using EG = EaGroup<K, NQ, PHYS, Real>;
    constexpr int NB = E::NB, NG = E::NG, GS = E::GS, NGRP = THREADS / GS;
    extern __shared__ __align__(128) char smem_raw[];
    const int tid = threadIdx.x, lane = tid % GS, grp = tid / GS;
    const unsigned gmask = GS >= 32 ? 0xFFFFFFFFu : (((1u << GS) - 1u) << ((tid & 31) / GS * GS));
    const int gbase = (tid & 31) - lane;
    {
        // the host sized the allocation from the same layout; refuse to run past it
        uint32_t dyn;
        asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
        if ((uint32_t)element_smem_bytes<K, NQ, PHYS, Real>(shape_bytes) > dyn) {
            if (tid == 0) atomicAdd(&a.status->timeout, 1u);
            return;
        }
    }
    Real* shape = (Real*)smem_raw;
    for (int k = tid; k < shape_bytes / 16; k += THREADS) ((int4*)shape)[k] = ((const int4*)shape_g)[k];
    char* base = smem_raw + pad16(shape_bytes);
    // tables of all groups first, so their strides keep the bank stagger of the tile kernel
    Real* tb = (Real*)(base + grp * EG::TB);
    char* xs = base + NGRP * EG::TB + grp * EG::XS;
    int32_t* nodes = (int32_t*)(base + NGRP * (EG::TB + EG::XS) + grp * EG::ND);
    uint16_t* cn = (uint16_t*)(base + NGRP * (EG::TB + EG::XS + EG::ND) + grp * EG::CN);
    if (lane < NG) cn[lane] = (uint16_t)lane;
    __syncthreads();
    const char* src = sizeof(Real) == 4 ? (const char*)a.xf6 : (const char*)a.xd3;
    const int64_t step = (int64_t)gridDim.x * NGRP;
    // node ids two cells ahead and coordinates one cell ahead, in registers (lanes < NG)
    const int64_t c0 = (int64_t)blockIdx.x * NGRP + grp;
    int nd_cur = 0, nd_next = 0;
    uint2 x_cur[3] = {}, x_next[3] = {};
    if (lane < NG) {
        if (c0 < sd.n_cells) {
            nd_cur = sd.conn[c0 * NG + lane];
            const uint2* p = (const uint2*)(src + (int64_t)nd_cur * NODE_BYTES);
            x_cur[0] = p[0]; x_cur[1] = p[1]; x_cur[2] = p[2];
        }
        if (c0 + step < sd.n_cells) nd_next = sd.conn[(c0 + step) * NG + lane];
    }
    for (int64_t c = c0; c < sd.n_cells; c += step) {
        int nd_after = 0;
        if (lane < NG) {
            nodes[lane] = nd_cur;
            uint2* d = (uint2*)(xs + lane * NODE_BYTES);
            d[0] = x_cur[0];
            d[1] = x_cur[1];
            d[2] = x_cur[2];
            if (c + step < sd.n_cells) {
                const uint2* p = (const uint2*)(src + (int64_t)nd_next * NODE_BYTES);
                x_next[0] = p[0]; x_next[1] = p[1]; x_next[2] = p[2];
            }
            if (c + 2 * step < sd.n_cells) nd_after = sd.conn[(c + 2 * step) * NG + lane];
        }
        __syncwarp(gmask);
        geometry_lanes<K, NQ, PHYS, Real>(a, sd, shape, (int)c, cn, xs, nodes, lane, gmask, gbase, tb);
        __syncwarp(gmask);
        if (lane < NB)
            cell_blocks<K, NQ, PHYS, Real, MODE>(a, sd, nullptr, nullptr, nullptr, 0, tb, shape, (int)c, lane, 0, NB,
                                                 (Real*)eo.ke + c * eo.ks[0], &eo);
        __syncwarp(gmask);  // the next cell overwrites the table and the coordinates
        nd_cur = nd_next;
        nd_next = nd_after;
        #pragma unroll
        for (int k = 0; k < 3; ++k) x_cur[k] = x_next[k];
    }
}

// ---------------------------------------------------------------------------------------
// element matrices of 27-node hexahedra (isotropic elasticity) on the tensor cores
// (tcgen05, kind::tf32). Per cell the blocks need only the Gram matrix of the scaled
// gradients, G[(i,a),(j,b)] = sum_q g_ia(q) g_jb(q) (g = sqrt(detJ w) grad N), since
// Ke[(i,a),(j,b)] = lam G[(i,a),(j,b)] + mu G[(i,b),(j,a)] + mu delta_ab sum_c G[(i,c),(j,c)]
// (threaded_assembly.jl:105-132 with C isotropic). G = A A^T with A the 81 x 27 matrix of
// gradient components (row m = 32 a + i, column = point): one M=128, N=96 MMA chain per
// product, K = 32 (27 points padded), accumulated in TMEM in FP32. TF32 keeps 10 mantissa
// bits, so A = hi + lo is split and G = hi hi^T + hi lo^T + lo hi^T (the lo lo^T term is
// below FP32 rounding). Operands live in shared memory in the K-major core-matrix layout
// without swizzle: (m, k) at (m%8)*16 + (k%4)*4 + (k/4)*128 + (m/8)*1024 bytes.
// 128 threads per cell:
//   - warp 3 maps the 27 points once (lane = point: J, s J^-1, the point weights), the next
//     cell's while the products run and warps 0-2 write this cell's element matrix (two
//     point-weight tables; warps 0-2 alone wait for the products and meet at a 96-thread
//     barrier);
//   - every warp forms gradients with lane = base function i over its quads of points and
//     writes them, split into tf32 hi and lo parts, straight into the operand rows 32 a + i
//     (16-byte stores of four points);
//   - warps 0-2 read back the rows of G (warp a = component a: TMEM lane 32 a + i) and write
//     the element matrix columns [j][t][i] of the two-phase scratch; warp 3 the load vector.
// Only the live rows (a < 3, i < 27) and points are rewritten per cell. The rest of the
// operands may hold stale values of the G exchange: they enter only rows and columns of the
// product that are never read.
// ---------------------------------------------------------------------------------------
constexpr int TC_OPERAND_BYTES = 128 * 32 * 4;  // one 128 x 32 tf32 operand
constexpr int TC_GS = 81;                        // row stride (floats) of the G exchange (odd: no bank conflicts)

constexpr int TC_JT_POINTS = 28;                 // 27 points and a zero pad point

struct TcLayout {
    int shape, tb0, tb1, xs, nodes, cn, jt, hi, lo, bytes;
};
__host__ __device__ inline TcLayout tc_layout(int shape_bytes) {
    using CT = CellTable<KIND_HEX27, 27, PHYS_ELASTIC, float>;
    TcLayout L;
    int o = 0;
    L.shape = o; o += pad16i(shape_bytes);
    // two cell tables (this cell's, the next cell's) of which only the point weights and the
    // cell factors are written, the gradients going to the operands: each table's base sits
    // CT::GRAD floats before those, over the shape tables
    if (o < CT::GRAD * 4) o = CT::GRAD * 4;
    L.tb0 = o - CT::GRAD * 4; o += pad16i((CT::SQ + 4) * 4);
    L.tb1 = o - CT::GRAD * 4; o += pad16i((CT::SQ + 4) * 4);
    L.xs = o; o += 8 * NODE_BYTES;
    L.nodes = o; o += 32;
    L.cn = o; o += 16;
    L.jt = o; o += TC_JT_POINTS * JT_STRIDE * 4;
    o = (o + 127) & ~127;
    L.hi = o; o += TC_OPERAND_BYTES;
    L.lo = o; o += TC_OPERAND_BYTES;
    L.bytes = o;
    return L;
}

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    // start address, leading byte offset (next core matrix along K) 128, stride byte offset
    // (next 8-row group) 1024, all in 16-byte units; bits 46-48 = 0b001; no swizzle
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, long long limit) {
    for (long long it = 0; it < limit; ++it) {
        uint32_t ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, float* r) {
    uint32_t v[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,"
        "%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
          "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
          "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]),
          "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    #pragma unroll
    for (int k = 0; k < 32; ++k) r[k] = __uint_as_float(v[k]);
}

// The rows of G of component AA (one warp, lane = function i) into the element matrix columns
// of one cell: Ke[(i,a),(j,b)] = lam G[(i,a),(j,b)] + mu G[(i,b),(j,a)] + mu delta_ab tr, with
// tr = sum_c G[(i,c),(j,c)]. The warp's own row comes from registers (g: G[(i,AA),(j,b)] at
// 32 b + j), the other components' rows from the exchange (G: row 32 c + i, TC_GS apart).
template <int AA, int NB, int JS>
__device__ __forceinline__ void tc_ke_rows(const float* __restrict__ G, const float* g, float lam, float mu, int i,
                                           float* __restrict__ out) {
    const float* Gi[3] = {G + i * TC_GS, G + (32 + i) * TC_GS, G + (64 + i) * TC_GS};
    #pragma unroll
    for (int j = 0; j < NB; ++j) {
        const float d0 = AA == 0 ? g[j] : Gi[0][j];
        const float d1 = AA == 1 ? g[32 + j] : Gi[1][NB + j];
        const float d2 = AA == 2 ? g[64 + j] : Gi[2][2 * NB + j];
        const float tr = d0 + d1 + d2;
        #pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float gab = g[32 * b + j];
            const float gba = b == AA ? gab : Gi[b][NB * AA + j];  // G[(i,b),(j,a)]
            float v = lam * gab + mu * gba;
            if (b == AA) v += mu * tr;
            out[j * JS + (b * 3 + AA) * NB + i] = v;
        }
    }
}

template <int PHYS>
__global__ void __launch_bounds__(128, 3) element_kernel_tc(const KernelArgs a, const SubDev sd, const float* __restrict__ shape_g,
                                                             int shape_bytes, const EaOut eo) {
    static_assert(PHYS == PHYS_ELASTIC, "the Gram-matrix form is isotropic elasticity");
    constexpr int K = KIND_HEX27, NQ = 27, NB = 27, NG = 8;
    using CT = CellTable<K, NQ, PHYS_ELASTIC, float>;
    constexpr ShapeQ SQL = shape_q(NB, NG, 3, 4);
    constexpr int JS = ea_col_values(NB, 3);
    static_assert(NB * 3 <= TC_GS && (NQ + 3) / 4 <= 7, "rows of the exchange; point quads 0-6 live, quad 7 pads");
    extern __shared__ __align__(128) char smem_raw[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ uint32_t tmem_base;
    const TcLayout L = tc_layout(shape_bytes);
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    {
        // the host sized the allocation from the same layout; refuse to run past it
        uint32_t dyn;
        asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
        if ((uint32_t)L.bytes > dyn) {
            if (tid == 0) atomicAdd(&a.status->timeout, 1u);
            return;
        }
    }
    float* shape = (float*)(smem_raw + L.shape);
    float* const tb0 = (float*)(smem_raw + L.tb0);
    float* const tb1 = (float*)(smem_raw + L.tb1);
    char* xs = smem_raw + L.xs;
    int32_t* nodes = (int32_t*)(smem_raw + L.nodes);
    uint16_t* cn = (uint16_t*)(smem_raw + L.cn);
    float* jt = (float*)(smem_raw + L.jt);
    float* G = (float*)(smem_raw + L.hi);  // the G exchange reuses the operands (96 x 81 floats)
    for (int k = tid; k < shape_bytes / 16; k += 128) ((int4*)shape)[k] = ((const int4*)shape_g)[k];
    if (tid < NG) cn[tid] = (uint16_t)tid;
    // the pad point's row of the Jacobian table and all of both operands start at zero
    for (int k = tid; k < TC_JT_POINTS * JT_STRIDE; k += 128) jt[k] = 0.f;
    for (int k = tid; k < 2 * TC_OPERAND_BYTES / 16; k += 128) ((float4*)(smem_raw + L.hi))[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t barp = (uint32_t)__cvta_generic_to_shared(&bar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(barp) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"((uint32_t)__cvta_generic_to_shared(&tmem_base))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tm = tmem_base;
    const uint32_t hi_s = (uint32_t)__cvta_generic_to_shared(smem_raw + L.hi);
    const uint32_t lo_s = (uint32_t)__cvta_generic_to_shared(smem_raw + L.lo);
    // D f32, A and B tf32, both K-major, N = 96, M = 128
    constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(96 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    const char* src = (const char*)a.xf6;
    bool failed = false;
    int it = 0;
    // Warp 3 maps the cells' points: the first cell's before the loop, every next one after
    // this cell's load vector, while the products run and warps 0-2 write this cell's element
    // matrix. Its lanes < NG
    // hold node ids two cells ahead and coordinates one cell ahead in registers, so neither
    // global round trip sits on the critical path.
    const int64_t G0 = gridDim.x;
    const bool nl = warp == 3 && lane < NG;
    int nd_cur = 0, nd_next = 0;
    uint2 x_cur[3] = {}, x_next[3] = {};
    if (nl) {
        if ((int64_t)blockIdx.x < sd.n_cells) {
            nd_cur = sd.conn[(int64_t)blockIdx.x * NG + lane];
            const uint2* p = (const uint2*)(src + (int64_t)nd_cur * NODE_BYTES);
            x_cur[0] = p[0]; x_cur[1] = p[1]; x_cur[2] = p[2];
        }
        if ((int64_t)blockIdx.x + G0 < sd.n_cells) nd_next = sd.conn[((int64_t)blockIdx.x + G0) * NG + lane];
    }
    // cell cc's nodes into shared memory, then its 27 points (lane = point): s J^-1 into jt,
    // point weights and cell factors into table tbc (warp 3 only)
    auto map_cell = [&](int64_t cc, float* tbc) {
        int nd_after = 0;
        __syncwarp();  // the previous cell's geometry has read the node data
        if (nl) {
            nodes[lane] = nd_cur;
            uint2* d = (uint2*)(xs + lane * NODE_BYTES);
            d[0] = x_cur[0];
            d[1] = x_cur[1];
            d[2] = x_cur[2];
            if (cc + G0 < sd.n_cells) {
                const uint2* p = (const uint2*)(src + (int64_t)nd_next * NODE_BYTES);
                x_next[0] = p[0]; x_next[1] = p[1]; x_next[2] = p[2];
            }
            if (cc + 2 * G0 < sd.n_cells) nd_after = sd.conn[(cc + 2 * G0) * NG + lane];
        }
        __syncwarp();
        geometry_lanes<K, NQ, PHYS_ELASTIC, float>(a, sd, shape, (int)cc, cn, xs, nodes, lane, 0xFFFFFFFFu, 0, tbc, 0, 0, true,
                                                    jt);
        nd_cur = nd_next;
        nd_next = nd_after;
        #pragma unroll
        for (int k = 0; k < 3; ++k) x_cur[k] = x_next[k];
    };
    if (warp == 3 && (int64_t)blockIdx.x < sd.n_cells) map_cell(blockIdx.x, tb0);
    __syncthreads();
    // byte offset of this lane's operand row 32 a + i for a = 0 (a component adds 4096)
    const int rowb = (lane & 7) * 16 + (lane >> 3) * 1024;
    for (int64_t c = blockIdx.x; c < sd.n_cells; c += gridDim.x, ++it) {
        const float* tbc = (it & 1) ? tb1 : tb0;
        // gradients g_i(q) = dN_i(q) s J^-1(q), lane = base function i, into the operands
        // (m, k) = (32 a + i, point); warp w takes the point quads w and w + 4 (point 27 pads)
        if (lane < NB) {
            for (int qq = warp; qq < 7; qq += 4) {
                float x[3][4];
                #pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const int q = 4 * qq + h;
                    float dN[3] = {0.f, 0.f, 0.f};
                    if (q < NQ) {
                        const float* Q = shape + q * SQL.qs + SQL.dn + 3 * lane;
                        dN[0] = Q[0]; dN[1] = Q[1]; dN[2] = Q[2];
                    }
                    const float* Jq = jt + q * JT_STRIDE;
                    const float4 j0 = *(const float4*)Jq, j1 = *(const float4*)(Jq + 4);
                    const float Ji[9] = {j0.x, j0.y, j0.z, j0.w, j1.x, j1.y, j1.z, j1.w, Jq[8]};
                    float g[3] = {0.f, 0.f, 0.f};
                    #pragma unroll
                    for (int b = 0; b < 3; ++b)
                        #pragma unroll
                        for (int cc = 0; cc < 3; ++cc) g[b] += dN[cc] * Ji[cc * 3 + b];
                    x[0][h] = g[0];
                    x[1][h] = g[1];
                    x[2][h] = g[2];
                }
                #pragma unroll
                for (int ca = 0; ca < 3; ++ca) {
                    float4 hv, lv;
                    float* hp = &hv.x;
                    float* lp = &lv.x;
                    #pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        uint32_t hb;
                        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hb) : "f"(x[ca][r]));
                        hp[r] = __uint_as_float(hb);
                        lp[r] = x[ca][r] - hp[r];
                    }
                    const int off = rowb + ca * 4096 + qq * 128;
                    *(float4*)(smem_raw + L.hi + off) = hv;
                    *(float4*)(smem_raw + L.lo + off) = lv;
                }
            }
            if (warp == 3) {
                // points 28-31 of the live rows (the exchange of G overwrote them)
                #pragma unroll
                for (int ca = 0; ca < 3; ++ca) {
                    const int off = rowb + ca * 4096 + 7 * 128;
                    *(float4*)(smem_raw + L.hi + off) = make_float4(0.f, 0.f, 0.f, 0.f);
                    *(float4*)(smem_raw + L.lo + off) = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // operand writes -> tensor core reads
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            #pragma unroll
            for (int prod = 0; prod < 3; ++prod) {
                const uint32_t as = prod == 2 ? lo_s : hi_s, bs = prod == 1 ? lo_s : hi_s;
                #pragma unroll
                for (int s = 0; s < 4; ++s) {
                    const uint64_t da = tc_desc(as + s * 256), db = tc_desc(bs + s * 256);
                    const uint32_t acc = (prod | s) ? 1u : 0u;
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tm),
                        "l"(da), "l"(db), "r"(IDESC), "r"(acc)
                        : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(barp) : "memory");
        }
        float* out = (float*)eo.ke + c * eo.ks[0];
        // warps 0-2 wait for the products and read TMEM; warp 3 reads none and goes on with the
        // load vector and the next cell's points (jt, the node data and the other table are
        // free once the operands are written)
        bool ok = true;
        float g[96];
        if (warp < 3) {
            ok = __all_sync(0xFFFFFFFFu, tc_wait(barp, (uint32_t)(it & 1), WAIT_LIMIT));
            if (ok) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // rows of G: warp a reads TMEM lanes 32 a .. 32 a + 31 (lane = function i)
                #pragma unroll
                for (int c0 = 0; c0 < 3; ++c0) tc_ld32(tm + ((uint32_t)(32 * warp) << 16) + (uint32_t)(32 * c0), g + 32 * c0);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (lane < NB) {
                    #pragma unroll
                    for (int b = 0; b < 3; ++b)
                        #pragma unroll
                        for (int j = 0; j < NB; ++j) G[(32 * warp + lane) * TC_GS + NB * b + j] = g[32 * b + j];
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            asm volatile("bar.sync 1, 96;" ::: "memory");  // warps 0-2: the rows of G exchanged
            if (ok && lane < NB && a.do_k) {
                const float lam = tbc[CT::GRAD + CT::SQ], mu = tbc[CT::GRAD + CT::SQ + 1];
                if (warp == 0) tc_ke_rows<0, NB, JS>(G, g, lam, mu, lane, out);
                else if (warp == 1) tc_ke_rows<1, NB, JS>(G, g, lam, mu, lane, out);
                else tc_ke_rows<2, NB, JS>(G, g, lam, mu, lane, out);
            }
        } else {
            // the load vector, fe[(i,a)] = b_a sum_q N_i(q) detJ w, then the next cell's points
            if (a.do_f && lane < NB) {
                const float* sq = tbc + CT::GRAD;
                float Fi = 0.f;
                #pragma unroll
                for (int q = 0; q < NQ; ++q) Fi += sq[q] * shape[q * SQL.qs + SQL.n + lane];
                #pragma unroll
                for (int aa = 0; aa < 3; ++aa) out[NB * JS + aa * NB + lane] = Fi * a.phys.body_f[aa];
            }
            if (c + G0 < sd.n_cells) map_cell(c + G0, (it & 1) ? tb0 : tb1);
        }
        if (__syncthreads_or(!ok)) {  // the next cell overwrites the operands and G; a lost MMA: all leave
            failed = true;
            break;
        }
    }
    if (failed) {
        // the MMAs of this cell did not report back: record it and wait (bounded) once more
        // before the operands and TMEM are released
        if (tid == 0) atomicAdd(&a.status->timeout, 1u);
        tc_wait(barp, (uint32_t)(it & 1), WAIT_LIMIT);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tm) : "memory");
}

}  // namespace fe
