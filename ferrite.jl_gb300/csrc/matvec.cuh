// matvec.cuh -- matrix-free product with element matrices, y (+)= sum_c A_c^T Ke_c A_c u: the
// consumer of the element-assembly output (Kes[cell, i, j] of
// docs/src/literate-howto/gpu_assembly.jl:265-303, which leaves the product itself to the user).
// Deterministic, without atomics, in two passes:
//   element_products (cells adjacent in memory, the how-to's Kes[ncells, nbf, nbf]): one
//     thread per cell, ye = Ke_c u_e with fused multiply-adds in the element precision
//     (J ascending), written to a scratch laid out [n][cells] per subdomain, so a warp's loads
//     and stores are consecutive cells; element_products_rows (one block per cell): one warp
//     per cell, the same chains, scratch [cells][n];
//   dof_gather: one thread per dof, y[d] (+)= its cells' ye entries in ascending cell order
//     (an incidence list built once on the host), summed in FP64.
// The result is bitwise that of the serial loop over cells in order.
#pragma once
#include <stdint.h>

namespace fe {

template <typename T>
struct MatvecPrec;
template <>
struct MatvecPrec<float> {
    static __device__ __forceinline__ float from(double v) { return __double2float_rn(v); }
    static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
};
template <>
struct MatvecPrec<double> {
    static __device__ __forceinline__ double from(double v) { return v; }
    static __device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
};

// ye[I * n_cells + k] = sum_J Ke_c(I, J) u[dofs[J * n_cells + k]], c = cells[k], accumulated as
// fma(Ke(I, J), u_J, acc) with J ascending from acc = 0. N = dofs per cell (compile time, so
// the accumulators stay in registers). The rows of a cell are split over S threads (warps
// wg*S .. wg*S + S-1 take the same 32 cells, part p rows [p*RP, p*RP + RP)), so that small grids
// still have enough threads to fill the machine without a long last wave.
template <typename T, int N, int S>
__global__ void __launch_bounds__(128) element_products(const T* __restrict__ ke, int64_t ks0, int64_t ks1, int64_t ks2,
                                                        const int32_t* __restrict__ cells, const int32_t* __restrict__ dofs,
                                                        int64_t n_cells, const double* __restrict__ u, T* __restrict__ ye) {
    static_assert(4 % S == 0, "a 128-thread block holds whole groups of S warps");
    constexpr int RP = (N + S - 1) / S;
    const int lane = threadIdx.x & 31;
    const int64_t wg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwg = ((int64_t)gridDim.x * blockDim.x) >> 5;  // a multiple of S
    const int i0 = (int)(wg % S) * RP;
    for (int64_t k = (wg / S) * 32 + lane; k < n_cells; k += (nwg / S) * 32) {
        const T* kc = ke + (int64_t)cells[k] * ks0;
        T acc[RP];
#pragma unroll
        for (int i = 0; i < RP; ++i) acc[i] = T(0);
        auto step = [&](int J) {
            const T uj = MatvecPrec<T>::from(u[dofs[(int64_t)J * n_cells + k]]);
            const T* col = kc + (int64_t)J * ks2;
#pragma unroll
            for (int i = 0; i < RP; ++i)
                if (i0 + i < N) acc[i] = MatvecPrec<T>::fma(__ldg(col + (int64_t)(i0 + i) * ks1), uj, acc[i]);
        };
        if constexpr (sizeof(T) == 8) {
            // the FP64 pipe is the bound; the unrolled form measured slower
#pragma unroll 1
            for (int J = 0; J < N; ++J) step(J);
        } else {
            // four J per step: their u and Ke loads do not depend on the chains, so they issue together
#pragma unroll 4
            for (int J = 0; J < N; ++J) step(J);
        }
#pragma unroll
        for (int i = 0; i < RP; ++i)
            if (i0 + i < N) ye[(int64_t)(i0 + i) * n_cells + k] = acc[i];
    }
}

// row parts per cell of element_products: float products are bound by memory latency and gain
// from more threads; double ones by the FP64 pipe (1/64 of the FP32 rate), where a split only
// repeats the u loads
template <typename T>
constexpr int products_split(int n) {
    return sizeof(T) == 8 ? 1 : (n >= 24 ? 4 : (n >= 12 ? 2 : 1));
}

// 16-byte loads of W consecutive elements (float4 / double2)
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    static constexpr int W = 4;
    static __device__ __forceinline__ void load(const float* p, float* v) {
        const float4 x = __ldg(reinterpret_cast<const float4*>(p));
        v[0] = x.x;
        v[1] = x.y;
        v[2] = x.z;
        v[3] = x.w;
    }
};
template <>
struct Vec16<double> {
    static constexpr int W = 2;
    static __device__ __forceinline__ void load(const double* p, double* v) {
        const double2 x = __ldg(reinterpret_cast<const double2*>(p));
        v[0] = x.x;
        v[1] = x.y;
    }
};

// The same products for layouts where a cell's matrix is one block (cells not adjacent in
// memory, e.g. Kes[c, I, J] row-major): one warp per cell, lane I owning rows I, I + 32, ...
// and running the same fma chain over J ascending, u_J broadcast by a shuffle from the lane
// that loaded it. A warp's cell block stays in L1 while the J loop walks it. dofs and ye are
// laid out [cells][N] here, so the per-cell loads and stores are contiguous.
// VEC: J contiguous (ks2 == 1) with 16-byte aligned rows, N a multiple of W: each lane loads W
// consecutive J of its row at once; the fma chain is unchanged.
template <typename T, int N, bool VEC>
__global__ void __launch_bounds__(256) element_products_rows(const T* __restrict__ ke, int64_t ks0, int64_t ks1, int64_t ks2,
                                                             const int32_t* __restrict__ cells, const int32_t* __restrict__ dofs,
                                                             int64_t n_cells, const double* __restrict__ u, T* __restrict__ ye) {
    constexpr int R = (N + 31) / 32;  // rows (and u values) per lane
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = w0; k < n_cells; k += nw) {  // warp-uniform
        const T* kc = ke + (int64_t)cells[k] * ks0;
        T ul[R], acc[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int J = lane + 32 * r;
            ul[r] = J < N ? MatvecPrec<T>::from(u[dofs[k * N + J]]) : T(0);
            acc[r] = T(0);
        }
#pragma unroll
        for (int jb = 0; jb < R; ++jb) {
            constexpr int last = N - 32 * (R - 1);
            const int jn = jb == R - 1 ? last : 32;
            if constexpr (VEC) {
                constexpr int W = Vec16<T>::W;
                static_assert(N % W == 0, "vector rows need N a multiple of W");
#pragma unroll 2
                for (int jj = 0; jj < jn; jj += W) {
                    T v[R][W];
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const int I = lane + 32 * r;
                        if (I < N) Vec16<T>::load(kc + (int64_t)I * ks1 + 32 * jb + jj, v[r]);
                    }
#pragma unroll
                    for (int w = 0; w < W; ++w) {
                        const T uj = __shfl_sync(0xffffffffu, ul[jb], jj + w);
#pragma unroll
                        for (int r = 0; r < R; ++r)
                            if (lane + 32 * r < N) acc[r] = MatvecPrec<T>::fma(v[r][w], uj, acc[r]);
                    }
                }
            } else {
#pragma unroll 8
                for (int jj = 0; jj < jn; ++jj) {
                    const T uj = __shfl_sync(0xffffffffu, ul[jb], jj);
                    const T* col = kc + (int64_t)(32 * jb + jj) * ks2;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const int I = lane + 32 * r;
                        if (I < N) acc[r] = MatvecPrec<T>::fma(__ldg(col + (int64_t)I * ks1), uj, acc[r]);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int I = lane + 32 * r;
            if (I < N) ye[k * N + I] = acc[r];
        }
    }
}

// y[d] = (fillzero ? 0 : y[d]) + sum over its incidences (ascending cell order) of (double) ye
template <typename T>
__global__ void __launch_bounds__(256) dof_gather(const T* __restrict__ ye, const int64_t* __restrict__ ptr,
                                                  const int32_t* __restrict__ inc, int64_t ndofs, int fillzero,
                                                  double* __restrict__ y) {
    for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < ndofs; d += (int64_t)gridDim.x * blockDim.x) {
        double acc = fillzero ? 0.0 : y[d];
        const int64_t e1 = ptr[d + 1];
        // up to 8 incidences' loads in flight, then their sums in order
        for (int64_t e = ptr[d]; e < e1; e += 8) {
            T v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = e + q < e1 ? ye[inc[e + q]] : T(0);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (e + q < e1) acc = __dadd_rn(acc, (double)v[q]);
        }
        y[d] = acc;
    }
}

}  // namespace fe
