// facet.cuh -- facet (Neumann) loads on the device: FacetValues reinit! per facet point
// (src/FEValues/FacetValues.jl:129-155) and f[celldofs] += sum_q (N_i t_a) dGamma
// (benchmark/helper.jl:331-348; hyperelasticity.jl:278-290), t = pressure n + traction. FP64
// throughout, each operation rounded separately in the reference's order (J accumulated over
// the geometric nodes, weighted normal from the facet's reference tangents, |wn| = sqrt of the
// squares summed in order), so the result matches a serial FP64 evaluation bit for bit.
#pragma once
#include <stdint.h>

#include "common.h"
#include "tile_kernel.cuh"

namespace fe {

constexpr int FACET_WARPS = 8;

struct FacetArgs {
    int64_t n;          // facets
    int nf, nqp, nb, ng, nc, dim;
    const double* x;    // node coordinates [n_nodes][dim]
    const int32_t* nodes;   // [n][ng] 0-based node ids of each facet's cell
    const int32_t* fnr;     // [n] 0-based local facet numbers
    const int32_t* cellid;  // [n] 0-based cell ids (errors)
    const double* w;    // [nf][nqp]
    const double* N;    // [nf][nqp][nb]
    const double* dM;   // [nf][nqp][ng][dim]
    const double* tang; // [nf][6]: reference tangents u, v of each facet
    double pressure, t[3];
    double* contrib;    // [n][nb nc]
    DevStatus* status;
};

__device__ __forceinline__ double dmadd(double acc, double a, double b) { return __dadd_rn(acc, __dmul_rn(a, b)); }

// one warp per facet: lanes = points compute dGamma and the unit normal, then lanes run over
// the cell's load entries (i, a)
__global__ void __launch_bounds__(32 * FACET_WARPS) facet_contrib(const FacetArgs A) {
    __shared__ double pt[FACET_WARPS][32][4];
    const int wp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int nbf = A.nb * A.nc;
    for (int64_t k = (int64_t)blockIdx.x * FACET_WARPS + wp; k < A.n; k += (int64_t)gridDim.x * FACET_WARPS) {
        const int f = A.fnr[k];
        if (lane < A.nqp) {
            const int q = lane;
            const double* dMq = A.dM + ((int64_t)f * A.nqp + q) * A.ng * A.dim;
            double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int j = 0; j < A.ng; ++j) {
                const double* xj = A.x + (int64_t)A.nodes[k * A.ng + j] * A.dim;
                for (int a = 0; a < A.dim; ++a)
                    for (int b = 0; b < A.dim; ++b) J[a][b] = dmadd(J[a][b], xj[a], dMq[j * A.dim + b]);
            }
            const double* u = A.tang + f * 6;
            const double* v = u + 3;
            double wn[3] = {0, 0, 0};
            if (A.dim == 2) {
                const double ju0 = dmadd(__dmul_rn(J[0][0], u[0]), J[0][1], u[1]);
                const double ju1 = dmadd(__dmul_rn(J[1][0], u[0]), J[1][1], u[1]);
                wn[0] = ju1;
                wn[1] = -ju0;
            } else {
                double ju[3], jv[3];
                for (int a = 0; a < 3; ++a) {
                    ju[a] = dmadd(dmadd(__dmul_rn(J[a][0], u[0]), J[a][1], u[1]), J[a][2], u[2]);
                    jv[a] = dmadd(dmadd(__dmul_rn(J[a][0], v[0]), J[a][1], v[1]), J[a][2], v[2]);
                }
                wn[0] = __dsub_rn(__dmul_rn(ju[1], jv[2]), __dmul_rn(ju[2], jv[1]));
                wn[1] = __dsub_rn(__dmul_rn(ju[2], jv[0]), __dmul_rn(ju[0], jv[2]));
                wn[2] = __dsub_rn(__dmul_rn(ju[0], jv[1]), __dmul_rn(ju[1], jv[0]));
            }
            const double nrm = __dsqrt_rn(dmadd(dmadd(__dmul_rn(wn[0], wn[0]), wn[1], wn[1]), wn[2], wn[2]));
            if (!(nrm > 0.0)) {
                record_detj(A.status, A.cellid[k], (float)nrm);
                pt[wp][q][0] = pt[wp][q][1] = pt[wp][q][2] = pt[wp][q][3] = 0.0;
            } else {
                pt[wp][q][0] = __dmul_rn(nrm, A.w[f * A.nqp + q]);
                for (int a = 0; a < 3; ++a) pt[wp][q][1 + a] = __ddiv_rn(wn[a], nrm);
            }
        }
        __syncwarp();
        for (int I = lane; I < nbf; I += 32) {
            const int i = I / A.nc, a = I - i * A.nc;
            double fe = 0.0;
            for (int q = 0; q < A.nqp; ++q) {
                const double t = A.nc == 1 ? A.pressure : __dadd_rn(__dmul_rn(A.pressure, pt[wp][q][1 + a]), A.t[a]);
                const double s = __dmul_rn(A.N[((int64_t)f * A.nqp + q) * A.nb + i], t);
                fe = dmadd(fe, s, pt[wp][q][0]);
            }
            A.contrib[k * nbf + I] = fe;
        }
        __syncwarp();
    }
}

// f[row] += the facets' entries for that dof, in facet order (assemble!(f, dofs, fe) per facet)
__global__ void __launch_bounds__(256) facet_gather(double* __restrict__ f, const double* __restrict__ contrib,
                                                    const int64_t* __restrict__ rptr, const int64_t* __restrict__ rows,
                                                    const int64_t* __restrict__ epos, int64_t nrows) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
        double v = f[rows[r]];
        for (int64_t e = rptr[r]; e < rptr[r + 1]; ++e) v = __dadd_rn(v, contrib[epos[e]]);
        f[rows[r]] = v;
    }
}

}  // namespace fe
