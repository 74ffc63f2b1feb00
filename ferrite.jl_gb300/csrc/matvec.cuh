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
// the N accumulators stay in registers).
template <typename T, int N>
__global__ void __launch_bounds__(128) element_products(const T* __restrict__ ke, int64_t ks0, int64_t ks1, int64_t ks2,
                                                        const int32_t* __restrict__ cells, const int32_t* __restrict__ dofs,
                                                        int64_t n_cells, const double* __restrict__ u, T* __restrict__ ye) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n_cells; k += (int64_t)gridDim.x * blockDim.x) {
        const T* kc = ke + (int64_t)cells[k] * ks0;
        T acc[N];
#pragma unroll
        for (int I = 0; I < N; ++I) acc[I] = T(0);
#pragma unroll 1
        for (int J = 0; J < N; ++J) {
            const T uj = MatvecPrec<T>::from(u[dofs[(int64_t)J * n_cells + k]]);
            const T* col = kc + (int64_t)J * ks2;
#pragma unroll
            for (int I = 0; I < N; ++I) acc[I] = MatvecPrec<T>::fma(__ldg(col + (int64_t)I * ks1), uj, acc[I]);
        }
#pragma unroll
        for (int I = 0; I < N; ++I) ye[(int64_t)I * n_cells + k] = acc[I];
    }
}

// The same products for layouts where a cell's matrix is one block (cells not adjacent in
// memory, e.g. Kes[c, I, J] row-major): one warp per cell, lane I owning rows I, I + 32, ...
// and running the same fma chain over J ascending, u_J broadcast by a shuffle from the lane
// that loaded it. A warp's cell block stays in L1 while the J loop walks it. dofs and ye are
// laid out [cells][N] here, so the per-cell loads and stores are contiguous.
template <typename T, int N>
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
        for (int64_t e = ptr[d]; e < ptr[d + 1]; ++e) acc = __dadd_rn(acc, (double)ye[inc[e]]);
        y[d] = acc;
    }
}

}  // namespace fe
