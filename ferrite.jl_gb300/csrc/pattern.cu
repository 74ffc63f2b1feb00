// pattern.cu -- allocate_matrix(dh) on the device (src/Dofs/sparsity_pattern.jl:223-253, 549,
// 951-991): the CSC pattern that couples every two dofs sharing a cell, plus the diagonal,
// rows ascending in every column. Same numbering assumptions as the host fe_sparsity_pattern:
// one field of n_components interleaved dofs per entity (dof d belongs to entity (d-1)/nc).
//
// Per entity: its neighbour entities are the union of the entities of its cells (and itself),
// sorted and unique; column (e, b) then holds nc rows per neighbour. One warp per entity
// gathers the candidates into shared memory, sorts them (bitonic), and counts (first pass) or
// writes (second pass) the distinct ones. Incidence lists and prefix sums are integer work,
// so the result does not depend on the order in which atomics fill the incidence lists.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "device_buffers.h"
#include "ferrite_gb300.h"
#include "plan.h"

namespace {

constexpr int PAT_WARPS = 8;        // warps (entities) per block
constexpr int PAT_CAP = 1024;       // candidate entities per entity (cells x entities per cell)
constexpr int SCAN_CHUNK = 2048;    // elements per block of the prefix sums

__global__ void count_incidence(const int32_t* __restrict__ ents, int64_t n, int32_t* __restrict__ cnt) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[ents[k]], 1);
}

// exclusive prefix sums of 32-bit counts into 64-bit offsets: per-block sums, one block scans
// the block sums, then every block scans its chunk
__global__ void __launch_bounds__(256) scan_blocks(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ bsum) {
    __shared__ int64_t red[256];
    const int64_t b0 = (int64_t)blockIdx.x * SCAN_CHUNK;
    int64_t s = 0;
    for (int k = threadIdx.x; k < SCAN_CHUNK; k += 256)
        if (b0 + k < n) s += in[b0 + k];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(1) scan_sums(int64_t* __restrict__ bsum, int64_t nb) {
    int64_t run = 0;
    for (int64_t k = 0; k < nb; ++k) {
        const int64_t v = bsum[k];
        bsum[k] = run;
        run += v;
    }
    bsum[nb] = run;
}

__global__ void __launch_bounds__(256) scan_apply(const int32_t* __restrict__ in, int64_t n, const int64_t* __restrict__ bsum,
                                                  int64_t* __restrict__ out) {
    __shared__ int64_t part[256];
    const int64_t b0 = (int64_t)blockIdx.x * SCAN_CHUNK;
    constexpr int PER = SCAN_CHUNK / 256;
    int64_t v[PER];
    int64_t s = 0;
    #pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int64_t k = b0 + threadIdx.x * PER + q;
        v[q] = k < n ? in[k] : 0;
        s += v[q];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = 1; w < 256; w <<= 1) {  // inclusive scan of the thread sums
        const int64_t t = (int)threadIdx.x >= w ? part[threadIdx.x - w] : 0;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    int64_t run = bsum[blockIdx.x] + part[threadIdx.x] - s;
    #pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int64_t k = b0 + threadIdx.x * PER + q;
        if (k < n) out[k] = run;
        run += v[q];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = bsum[gridDim.x];
}

__global__ void fill_incidence(const int32_t* __restrict__ ents, const int32_t* __restrict__ slot_cell, int64_t n,
                               int64_t* __restrict__ cursor, int32_t* __restrict__ ecell) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        ecell[atomicAdd((unsigned long long*)&cursor[ents[k]], 1ull)] = slot_cell[k];
}

// the sorted distinct neighbour entities of entity e in buf (shared, PAT_CAP); returns their
// count, or -1 if the candidates exceed the buffer
__device__ int neighbours(int64_t e, const int64_t* __restrict__ eptr, const int32_t* __restrict__ ecell,
                          const int64_t* __restrict__ cstart, const int32_t* __restrict__ cnb, const int32_t* __restrict__ ents,
                          int32_t* buf, int lane) {
    // candidates: e itself, then the entities of its cells
    int n = 1;
    if (lane == 0) buf[0] = (int32_t)e;
    for (int64_t t = eptr[e]; t < eptr[e + 1]; ++t) {
        const int32_t c = ecell[t];
        const int nb = cnb[c];
        if (n + nb > PAT_CAP) return -1;
        const int64_t s0 = cstart[c];
        for (int i = lane; i < nb; i += 32) buf[n + i] = ents[s0 + i];
        n += nb;
    }
    int P = 32;
    while (P < n) P <<= 1;
    for (int i = n + lane; i < P; i += 32) buf[i] = 0x7FFFFFFF;
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < P; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const int32_t a = buf[i], b = buf[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        buf[i] = b;
                        buf[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    // compact the distinct values to the front, in order; a chunk's predecessor values come
    // from registers (the slots before it may already hold compacted values)
    int run = 0;
    int32_t carry = 0;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        const int32_t v = i < n ? buf[i] : 0x7FFFFFFF;
        int32_t prev = __shfl_up_sync(0xFFFFFFFFu, v, 1);
        if (lane == 0) prev = carry;
        carry = __shfl_sync(0xFFFFFFFFu, v, 31);
        const bool keep = i < n && (i == 0 || v != prev);
        const unsigned m = __ballot_sync(0xFFFFFFFFu, keep);
        __syncwarp();
        if (keep) buf[run + __popc(m & ((1u << lane) - 1u))] = v;
        run += __popc(m);
        __syncwarp();
    }
    return run;
}

__global__ void __launch_bounds__(32 * PAT_WARPS) count_neighbours(int64_t ne, const int64_t* __restrict__ eptr,
                                                                  const int32_t* __restrict__ ecell, const int64_t* __restrict__ cstart,
                                                                  const int32_t* __restrict__ cnb, const int32_t* __restrict__ ents,
                                                                  int32_t* __restrict__ nnb, int* __restrict__ overflow) {
    __shared__ int32_t sbuf[PAT_WARPS][PAT_CAP];
    const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (int64_t e = (int64_t)blockIdx.x * PAT_WARPS + w; e < ne; e += (int64_t)gridDim.x * PAT_WARPS) {
        const int k = neighbours(e, eptr, ecell, cstart, cnb, ents, sbuf[w], lane);
        if (lane == 0) {
            nnb[e] = k < 0 ? 0 : k;
            if (k < 0) atomicExch(overflow, 1);
        }
        __syncwarp();
    }
}

// column (e, b): rows nc r + a + 1 for the neighbours r of e (ascending) and a < nc
__global__ void __launch_bounds__(32 * PAT_WARPS) fill_rows(int64_t ne, int nc, const int64_t* __restrict__ eptr,
                                                           const int32_t* __restrict__ ecell, const int64_t* __restrict__ cstart,
                                                           const int32_t* __restrict__ cnb, const int32_t* __restrict__ ents,
                                                           const int64_t* __restrict__ roff, int64_t* __restrict__ rowval,
                                                           int* __restrict__ overflow) {
    __shared__ int32_t sbuf[PAT_WARPS][PAT_CAP];
    const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (int64_t e = (int64_t)blockIdx.x * PAT_WARPS + w; e < ne; e += (int64_t)gridDim.x * PAT_WARPS) {
        const int k = neighbours(e, eptr, ecell, cstart, cnb, ents, sbuf[w], lane);
        if (k < 0) {
            if (lane == 0) atomicExch(overflow, 1);
            continue;
        }
        const int64_t L = (int64_t)nc * k;
        int64_t* out = rowval + (int64_t)nc * nc * roff[e];
        for (int b = 0; b < nc; ++b)
            for (int64_t q = lane; q < L; q += 32) {
                const int t = (int)(q / nc), a = (int)(q - (int64_t)t * nc);
                out[b * L + q] = (int64_t)sbuf[w][t] * nc + a + 1;
            }
        __syncwarp();
    }
}

__global__ void make_colptr(int64_t ne, int nc, const int64_t* __restrict__ roff, const int32_t* __restrict__ nnb,
                            int64_t* __restrict__ colptr) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x)
        for (int b = 0; b < nc; ++b) colptr[e * nc + b] = 1 + (int64_t)nc * nc * roff[e] + (int64_t)b * nc * nnb[e];
    if (blockIdx.x == 0 && threadIdx.x == 0) colptr[ne * nc] = 1 + (int64_t)nc * nc * roff[ne];
}

bool device_memory(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

cudaError_t scan(const int32_t* in, int64_t n, int64_t* out, fe::DeviceBuffers& B) {
    const int64_t nb = std::max<int64_t>(1, (n + SCAN_CHUNK - 1) / SCAN_CHUNK);
    int64_t* bsum = nullptr;
    cudaError_t e = B.alloc(&bsum, (size_t)nb + 1);
    if (e != cudaSuccess) return e;
    scan_blocks<<<(unsigned)nb, 256>>>(in, n, bsum);
    scan_sums<<<1, 1>>>(bsum, nb);
    scan_apply<<<(unsigned)nb, 256>>>(in, n, bsum, out);
    return cudaGetLastError();
}

}  // namespace

namespace {

// ---------------------------------------------------------------------------------------
// The index map of a device-resident pattern (the device half of fe_create for a
// CuSparseMatrixCSC-style pattern; the host form is the end of build_problem in plan.cpp).
// ---------------------------------------------------------------------------------------
// Per dof entity n: its nc columns have the same rows, the rows come in entity blocks of nc
// consecutive dofs starting at a multiple of nc, and the blocks ascend. The smallest failing
// column (1-based) goes to bad.
__global__ void pattern_blocked(const int64_t* __restrict__ cp, const int64_t* __restrict__ rv, int64_t ne, int nc,
                                int64_t ndofs, unsigned long long* __restrict__ bad) {
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < ne; n += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c0 = cp[nc * n] - 1, L = cp[nc * n + 1] - cp[nc * n];
        bool b = (L % nc) != 0;
        for (int c = 1; c < nc && !b; ++c) {
            const int64_t cb = cp[nc * n + c] - 1;
            if (cp[nc * n + c + 1] - cp[nc * n + c] != L) { b = true; break; }
            for (int64_t k = 0; k < L; ++k)
                if (rv[cb + k] != rv[c0 + k]) { b = true; break; }
        }
        for (int64_t k = 0; k < L && !b; k += nc) {
            const int64_t r0 = rv[c0 + k];
            if (r0 < 1 || r0 > ndofs || (r0 - 1) % nc) { b = true; break; }
            if (k && rv[c0 + k - nc] >= r0) { b = true; break; }
            for (int a = 1; a < nc; ++a)
                if (rv[c0 + k + a] != r0 + a) { b = true; break; }
        }
        if (b) atomicMin(bad, (unsigned long long)(n * nc + 1));
    }
}

// Per (cell, column function j) of one subdomain, for every row function i: the rank of row
// entity e_i among column entity e_j's row entities (binary search of the ascending rows; the
// host's merge walk over the sorted entities finds the same position), miss where the column
// has no such row, and over set when a rank reaches the table type's limit.
template <typename RT>
__global__ void entity_ranks(const int64_t* __restrict__ cp, const int64_t* __restrict__ rv, const int32_t* __restrict__ ents,
                             int64_t n_cells, int nb, int nc, int64_t miss, int64_t limit, RT* __restrict__ out,
                             int* __restrict__ over) {
    const int64_t total = n_cells * nb;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = q / nb;
        const int j = (int)(q - k * nb);
        const int32_t* e = ents + k * nb;
        const int64_t n = e[j];
        const int64_t c0 = cp[nc * n] - 1, Le = (cp[nc * n + 1] - cp[nc * n]) / nc;
        for (int i = 0; i < nb; ++i) {
            const int64_t want = (int64_t)e[i] * nc + 1;
            int64_t lo = 0, hi = Le;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (rv[c0 + nc * mid] < want) lo = mid + 1;
                else hi = mid;
            }
            int64_t r = miss;
            if (lo < Le && rv[c0 + nc * lo] == want && lo < 0xFFFF) r = lo;
            if (r != miss && r >= limit) *over = 1;
            out[q * nb + i] = (RT)(r >= limit ? miss : r);
        }
    }
}

}  // namespace

namespace fe {

int device_index_map(HostProblem& hp, const int64_t* cp_dev, const int64_t* rv_dev, Error& err) {
    const int nc = hp.nc;
    DeviceBuffers B;
    unsigned long long* d_bad;
    int* d_over;
    auto cuda_err = [&](cudaError_t e) {
        err.code = FE_ERR_CUDA;
        err.msg = std::string("device index map: ") + cudaGetErrorString(e);
        return FE_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = B.alloc(&d_bad, 1)) != cudaSuccess || (e = B.alloc(&d_over, 1)) != cudaSuccess) return cuda_err(e);
    if ((e = cudaMemset(d_bad, 0xFF, sizeof(unsigned long long))) != cudaSuccess) return cuda_err(e);
    int dev = 0, n_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    const unsigned grid = (unsigned)std::max(1, n_sm * 8);
    pattern_blocked<<<grid, 256>>>(cp_dev, rv_dev, hp.n_ent, nc, hp.ndofs, d_bad);
    unsigned long long bad = 0;
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaMemcpy(&bad, d_bad, 8, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_err(e);
    if (bad != ~0ull) {
        err.col = (int64_t)bad;
        err.code = FE_ERR_UNSUPPORTED;
        err.msg = "sparsity pattern is not blocked by dof entity (all components coupled)";
        return FE_ERR_UNSUPPORTED;
    }
    for (HostSub& hs : hp.subs) {
        const int nb = hs.nb;
        const size_t n_rank = (size_t)hs.n_cells * nb * nb;
        int32_t* d_ents;
        uint8_t* d_r8;
        if ((e = B.upload(&d_ents, hs.ents.data(), hs.ents.size())) != cudaSuccess || (e = B.alloc(&d_r8, n_rank)) != cudaSuccess ||
            (e = cudaMemset(d_over, 0, sizeof(int))) != cudaSuccess)
            return cuda_err(e);
        entity_ranks<uint8_t><<<grid, 256>>>(cp_dev, rv_dev, d_ents, hs.n_cells, nb, nc, 255, 255, d_r8, d_over);
        int over = 0;
        if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaMemcpy(&over, d_over, 4, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_err(e);
        if (!over) {
            hs.wide_rank = false;
            hs.rank8.resize(n_rank);
            if ((e = cudaMemcpy(hs.rank8.data(), d_r8, n_rank, cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda_err(e);
        } else {
            B.release(d_r8);
            uint16_t* d_r16;
            if ((e = B.alloc(&d_r16, n_rank)) != cudaSuccess) return cuda_err(e);
            entity_ranks<uint16_t><<<grid, 256>>>(cp_dev, rv_dev, d_ents, hs.n_cells, nb, nc, 0xFFFF, 0xFFFF, d_r16, d_over);
            hs.wide_rank = true;
            decltype(hs.rank8)().swap(hs.rank8);
            hs.rank16.resize(n_rank);
            if ((e = cudaGetLastError()) != cudaSuccess ||
                (e = cudaMemcpy(hs.rank16.data(), d_r16, n_rank * 2, cudaMemcpyDeviceToHost)) != cudaSuccess)
                return cuda_err(e);
        }
        B.release(d_ents);
    }
    return FE_OK;
}

}  // namespace fe

extern "C" {

int fe_sparsity_pattern_device(const fe_grid_desc* grid, int32_t n_sub, const fe_subdomain_desc* subs, const fe_dof_desc* dofs,
                               int64_t* colptr, int64_t* rowval, int64_t* nnz) {
    if (!grid || !subs || !dofs || !colptr || !nnz || n_sub < 1) return FE_ERR_ARG;
    const int nc = subs[0].n_components;
    const int64_t nd = dofs->ndofs;
    if (nc < 1 || nd % nc) return FE_ERR_UNSUPPORTED;
    const int64_t ne = nd / nc;
    if (ne >= INT32_MAX) return FE_ERR_UNSUPPORTED;
    // per cell of every subdomain: its entities (from the first component of each base
    // function's dofs), where they start, how many
    int64_t n_slots = 0, n_cells = 0;
    std::vector<int32_t> nbs(n_sub);
    for (int s = 0; s < n_sub; ++s) {
        int32_t nb, ng, rdim;
        if (subs[s].n_components != nc || fe::kind_of(subs[s].cell_type, subs[s].ip_order, nb, ng, rdim) < 0)
            return FE_ERR_UNSUPPORTED;
        if (nb > 255) return FE_ERR_UNSUPPORTED;
        nbs[s] = nb;
        n_slots += subs[s].n_cells * nb;
        n_cells += subs[s].n_cells;
    }
    if (n_slots >= INT32_MAX || n_cells >= INT32_MAX) return FE_ERR_UNSUPPORTED;
    std::vector<int32_t> ents((size_t)n_slots), slot_cell((size_t)n_slots), cnb((size_t)n_cells);
    std::vector<int64_t> cstart((size_t)n_cells);
    int bad = 0;
    {
        int64_t slot0 = 0, cell0 = 0;
        for (int s = 0; s < n_sub; ++s) {
            const int nb = nbs[s];
            const int64_t n = subs[s].n_cells;
#pragma omp parallel for schedule(static) reduction(| : bad)
            for (int64_t k = 0; k < n; ++k) {
                const int64_t c = subs[s].cellset[k] - 1;
                if (c < 0 || c >= grid->n_cells) { bad = 1; continue; }
                const int64_t* cd = dofs->cell_dofs + dofs->cell_dofs_offset[c] - 1;
                const int64_t gc = cell0 + k, s0 = slot0 + k * nb;
                cstart[gc] = s0;
                cnb[gc] = nb;
                for (int i = 0; i < nb; ++i) {
                    const int64_t d = cd[i * nc];
                    if (d < 1 || d > nd || (d - 1) % nc) { bad = 1; break; }
                    ents[s0 + i] = (int32_t)((d - 1) / nc);
                    slot_cell[s0 + i] = (int32_t)gc;
                }
            }
            slot0 += n * nb;
            cell0 += n;
        }
    }
    if (bad) return FE_ERR_UNSUPPORTED;
    fe::DeviceBuffers B;
    int32_t *d_ents, *d_slot_cell, *d_cnb, *d_cnt, *d_ecell, *d_nnb;
    int64_t *d_cstart, *d_eptr, *d_cursor, *d_roff, *d_colptr;
    int* d_over;
    cudaError_t e = cudaSuccess;
#define PK(x)                                 \
    do {                                      \
        if ((e = (x)) != cudaSuccess) return FE_ERR_CUDA; \
    } while (0)
    PK(B.alloc(&d_ents, (size_t)n_slots));
    PK(B.alloc(&d_slot_cell, (size_t)n_slots));
    PK(B.alloc(&d_cnb, (size_t)n_cells));
    PK(B.alloc(&d_cstart, (size_t)n_cells));
    PK(B.alloc(&d_cnt, (size_t)ne));
    PK(B.alloc(&d_eptr, (size_t)ne + 1));
    PK(B.alloc(&d_cursor, (size_t)ne + 1));
    PK(B.alloc(&d_ecell, (size_t)n_slots));
    PK(B.alloc(&d_nnb, (size_t)ne));
    PK(B.alloc(&d_roff, (size_t)ne + 1));
    PK(B.alloc(&d_over, 1));
    PK(cudaMemcpy(d_ents, ents.data(), ents.size() * 4, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(d_slot_cell, slot_cell.data(), slot_cell.size() * 4, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(d_cnb, cnb.data(), cnb.size() * 4, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(d_cstart, cstart.data(), cstart.size() * 8, cudaMemcpyHostToDevice));
    PK(cudaMemset(d_cnt, 0, (size_t)ne * 4));
    PK(cudaMemset(d_over, 0, 4));
    int dev = 0, n_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    const unsigned grid1 = (unsigned)std::max(1, n_sm * 8);
    if (n_slots) count_incidence<<<grid1, 256>>>(d_ents, n_slots, d_cnt);
    PK(scan(d_cnt, ne, d_eptr, B));
    PK(cudaMemcpy(d_cursor, d_eptr, ((size_t)ne + 1) * 8, cudaMemcpyDeviceToDevice));
    if (n_slots) fill_incidence<<<grid1, 256>>>(d_ents, d_slot_cell, n_slots, d_cursor, d_ecell);
    const unsigned grid2 = (unsigned)std::min<int64_t>((ne + PAT_WARPS - 1) / PAT_WARPS, (int64_t)n_sm * 64);
    count_neighbours<<<grid2, 32 * PAT_WARPS>>>(ne, d_eptr, d_ecell, d_cstart, d_cnb, d_ents, d_nnb, d_over);
    PK(scan(d_nnb, ne, d_roff, B));
    int over = 0;
    PK(cudaMemcpy(&over, d_over, 4, cudaMemcpyDeviceToHost));
    if (over) return FE_ERR_UNSUPPORTED;  // an entity with more candidate neighbours than the buffer
    // colptr (1-based), in place if the caller's array is device memory
    const bool cp_dev = device_memory(colptr);
    if (cp_dev) d_colptr = colptr;
    else PK(B.alloc(&d_colptr, (size_t)nd + 1));
    make_colptr<<<grid1, 256>>>(ne, nc, d_roff, d_nnb, d_colptr);
    int64_t total = 0;
    PK(cudaMemcpy(&total, d_colptr + nd, 8, cudaMemcpyDeviceToHost));
    *nnz = total - 1;
    if (!cp_dev) PK(cudaMemcpy(colptr, d_colptr, ((size_t)nd + 1) * 8, cudaMemcpyDeviceToHost));
    if (!rowval) return FE_OK;
    const bool rv_dev = device_memory(rowval);
    int64_t* d_rowval = rowval;
    if (!rv_dev) PK(B.alloc(&d_rowval, (size_t)*nnz));
    fill_rows<<<grid2, 32 * PAT_WARPS>>>(ne, nc, d_eptr, d_ecell, d_cstart, d_cnb, d_ents, d_roff, d_rowval, d_over);
    PK(cudaGetLastError());
    if (!rv_dev) PK(cudaMemcpy(rowval, d_rowval, (size_t)*nnz * 8, cudaMemcpyDeviceToHost));
    PK(cudaDeviceSynchronize());
    PK(cudaMemcpy(&over, d_over, 4, cudaMemcpyDeviceToHost));
#undef PK
    return over ? FE_ERR_UNSUPPORTED : FE_OK;
}

}  // extern "C"
