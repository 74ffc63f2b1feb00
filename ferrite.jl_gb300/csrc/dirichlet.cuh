// dirichlet.cuh -- Dirichlet constraints on the assembled CSC matrix: apply!(K, f, ch) and
// apply_zero!(K, f, ch) of src/Dofs/ConstraintHandler.jl:711-744 (device counterpart
// ext/FerriteKAExt/constraints.jl:40-148). Deterministic and without atomics: the host works
// out once, from the pattern, every nzval entry each step touches (the diagonal positions,
// the entries to zero, and per row the prescribed-column entries of f -= K g), so a call
// reads and writes only those entries instead of scanning all of nzval and rowval.
#pragma once
#include <stdint.h>

namespace fe {

constexpr int DIAG_BLOCKS = 256;  // fixed partition of the meandiag sum: the same bits on every device

// meandiag (ConstraintHandler.jl:944-955), first level: sums of |K[i, i]| over a fixed
// partition of the dofs, each reduced in a fixed order
__global__ void __launch_bounds__(256) meandiag_partial(const double* __restrict__ nz, const int64_t* __restrict__ diag, int64_t n,
                                                        double* __restrict__ part) {
    __shared__ double red[256];
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t b0 = (int64_t)blockIdx.x * chunk;
    const int64_t b1 = b0 + chunk < n ? b0 + chunk : n;
    double s = 0.0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += 256) {
        const int64_t j = diag[i];
        if (j >= 0) s += fabs(nz[j]);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// second level: m = (sum of the partial sums) / n
__global__ void __launch_bounds__(256) meandiag_final(const double* __restrict__ part, int nb, int64_t n, double* __restrict__ m) {
    __shared__ double red[256];
    double s = 0.0;
    for (int k = threadIdx.x; k < nb; k += 256) s += part[k];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *m = red[0] / (double)n;
}

// f -= K g over the prescribed columns (add_inhomogeneities_csc!, ConstraintHandler.jl:752-767):
// one thread per row that has entries in prescribed columns; its entries in the order of the
// prescribed dofs, each a separate multiply and subtract as in the reference, skipping g = 0
__global__ void __launch_bounds__(256) apply_rows(double* __restrict__ f, const double* __restrict__ nz, const int64_t* __restrict__ rptr,
                                                  const int64_t* __restrict__ rows, const int64_t* __restrict__ epos,
                                                  const int32_t* __restrict__ epi, const double* __restrict__ g, int64_t nrows) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nrows; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = rows[k];
        double acc = f[r];
        for (int64_t e = rptr[k]; e < rptr[k + 1]; ++e) {
            const double v = g[epi[e]];
            if (v != 0.0) acc = __dsub_rn(acc, __dmul_rn(v, nz[epos[e]]));
        }
        f[r] = acc;
    }
}

// zero_out_columns! and zero_out_rows! (ConstraintHandler.jl:931-949): the listed entries
__global__ void __launch_bounds__(256) apply_zero_entries(double* __restrict__ nz, const int64_t* __restrict__ pos, int64_t n) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) nz[pos[k]] = 0.0;
}

// K[d, d] = m, f[d] = g_d m (0 m for apply_zero!) (ConstraintHandler.jl:735-742)
__global__ void __launch_bounds__(256) apply_diag(double* __restrict__ nz, double* __restrict__ f, const int64_t* __restrict__ dpos,
                                                  const int64_t* __restrict__ pd0, const double* __restrict__ g,
                                                  const double* __restrict__ m, int64_t np, int applyzero) {
    const double mv = *m;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < np; k += (int64_t)gridDim.x * blockDim.x) {
        nz[dpos[k]] = mv;
        if (f) f[pd0[k]] = __dmul_rn(applyzero ? 0.0 : g[k], mv);
    }
}

}  // namespace fe
