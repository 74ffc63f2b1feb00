// api.cu -- the extern "C" entry points declared in include/ferrite_gb300.h.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "device_buffers.h"
#include "ferrite_gb300.h"
#include "plan.h"
#include "registry.h"
#include "adjoint.cuh"
#include "dirichlet.cuh"
#include "facet.cuh"
#include "matvec.cuh"
#include "tile_kernel.cuh"

using namespace fe;

namespace {

struct Registries {
    std::vector<KernelEntry> tiles;
    std::vector<ElemEntry> elems;
};

const Registries& registries() {
    static Registries reg;
    static std::once_flag once;
    std::call_once(once, [] {
        register_heat(reg.tiles, reg.elems);
        register_elastic(reg.tiles, reg.elems);
        register_neo(reg.tiles, reg.elems);
    });
    return reg;
}

const std::vector<KernelEntry>& registry() { return registries().tiles; }

const ElemEntry* find_elem(int kind, int nq, int phys, bool fp64) {
    for (const ElemEntry& e : registries().elems)
        if (e.kind == kind && e.nq == nq && e.phys == phys && e.fp64 == (int)fp64) return &e;
    return nullptr;
}

const std::vector<AdjEntry>& adj_registry() {
    static std::vector<AdjEntry> reg;
    static std::once_flag once;
    std::call_once(once, [] { register_adjoint(reg); });
    return reg;
}

__global__ void to_float_kernel(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = (float)in[k];
}

bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Page-locked host memory: the device address the kernels reach it by (its mapping), else
// nullptr. Kernels then store into host memory directly, overlapping the transfer with the
// assembly instead of staging it and copying afterwards.
void* pinned_device_alias(void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

}  // namespace

struct fe_handle {
    HostProblem hp;
    Plan plan;
    DeviceBuffers mem;  // every device buffer of the handle
    KernelArgs base{};
    // staged reference tables (one block per subdomain), float and double
    float* shape_f = nullptr;
    double* shape_d = nullptr;
    int shape_bytes[2] = {0, 0}, shape_off1[2] = {0, 0}, shape_off2[2] = {0, 0};
    DevStatus* status_d = nullptr;
    DevStatus* status_h = nullptr;  // pinned
    // staging buffers for host-pointer calls
    double* nz_stage = nullptr;
    double* f_stage = nullptr;
    double* u_stage = nullptr;
    double* scale_stage = nullptr;
    float* u_f = nullptr;
    float* scale_f = nullptr;
    // adjoint: node -> (cell, geometric node) rows in cell order, per-row contributions,
    // staging for host-pointer calls
    int64_t adj_rows = 0;
    int64_t* adj_ptr = nullptr;
    int32_t* adj_row_ids = nullptr;
    void* adj_contrib = nullptr;
    double* lam_stage = nullptr;
    float* lam_f = nullptr;
    double* dscale_stage = nullptr;
    double* drho_stage = nullptr;
    double* dX_stage = nullptr;
    cudaStream_t last_stream = 0;
    int pending = 0;  // an FE_ASYNC assembly whose status has not been read
    // CUDA graphs of captured assembly sequences (fe_graph_capture)
    int capturing = 0;
    cudaStream_t cap_stream = 0;
    std::vector<std::pair<cudaGraph_t, cudaGraphExec_t>> graphs;
    fe_error_info last{};
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_events;  // recorded, unread
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_pool;    // free for reuse
    int64_t flagged = 0;
    double create_seconds = 0;
    int device = 0;
    int32_t stage_cap = 0;  // staging values per tile the current plan was built with
    int max_smem = 0, n_sm = 0;      // device attributes (read once)
    const void* fitted_fn = nullptr;  // kernel and form (two-phase subdomains) the plan was last fitted to
    unsigned fitted_mask = 0;
    bool plan_pinned = false;         // staging capacity set by the caller or the autotuner
    // form chosen by fe_autotune (bit s: subdomain s two-phase) for its physics and precision,
    // used when a call names no form; force_mask overrides everything while the tuner times
    bool tuned_valid = false;
    int32_t tuned_phys = 0, tuned_prec = 0;
    unsigned tuned_mask = 0;
    bool force_on = false;
    unsigned force_mask = 0;
    const void* occ_fn = nullptr;    // occupancy of the last launch configuration
    int occ_smem = -1, occ_per_sm = 1;
    int accumulate_status = 0;       // a pending FE_ASYNC assembly's status is still being collected
    void* ea_buf = nullptr;          // element-matrix scratch of the two-phase form (grown on demand)
    size_t ea_bytes = 0;

    template <typename T>
    cudaError_t alloc(T** p, size_t count) {
        return mem.alloc(p, count);
    }
    void release(void* p) { mem.release(p); }
    template <typename T>
    cudaError_t upload(T** p, const T* src, size_t count) {
        return mem.upload(p, src, count);
    }
    ~fe_handle() {
        for (auto& g : graphs) {
            if (g.second) cudaGraphExecDestroy(g.second);
            if (g.first) cudaGraphDestroy(g.first);
        }
        for (auto& e : prof_events) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
        for (auto& e : prof_pool) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
        if (status_h) cudaFreeHost(status_h);
    }
};

namespace {

thread_local fe_error_info g_create_error{};

int set_error(fe_handle* h, int code, const std::string& msg, int64_t cell = 0, double detJ = 0, int64_t row = 0,
              int64_t col = 0) {
    if (!h) return code;
    h->last.code = code;
    h->last.cell = cell;
    h->last.detJ = detJ;
    h->last.row = row;
    h->last.col = col;
    std::snprintf(h->last.message, sizeof(h->last.message), "%s", msg.c_str());
    return code;
}

int cuda_fail(fe_handle* h, cudaError_t e, const char* what) {
    const int code = (e == cudaErrorMemoryAllocation) ? FE_ERR_OOM : FE_ERR_CUDA;
    return set_error(h, code, std::string(what) + ": " + cudaGetErrorString(e));
}

// Read the device status of the last assembly and translate it into an FE_* code.
int finish_status(fe_handle* h) {
    const DevStatus& st = *h->status_h;
    h->flagged = st.flagged;
    h->pending = 0;
    h->accumulate_status = 0;
    if (st.timeout) return set_error(h, FE_ERR_CUDA, "a tile gave up: table copy timed out or shared memory too small");
    if (st.detj_key != ~0ull) {
        const int64_t cell = (int64_t)(st.detj_key >> 32) + 1;
        uint32_t bits = (uint32_t)(st.detj_key & 0xFFFFFFFFu);
        float dj;
        std::memcpy(&dj, &bits, 4);
        char buf[160];
        std::snprintf(buf, sizeof buf, "det(J) is not positive: det(J) = %g in cell %lld", (double)dj, (long long)cell);
        return set_error(h, FE_ERR_DETJ, buf, cell, dj);
    }
    if (st.miss_key != ~0ull) {
        const int64_t cell = (int64_t)(st.miss_key >> 32) + 1;
        const int I = (int)((st.miss_key >> 16) & 0xFFFF), J = (int)(st.miss_key & 0xFFFF);
        const int64_t* cd = h->hp.cell_dofs.data() + h->hp.cell_dofs_off[cell - 1] - 1;
        const int64_t row = cd[I], col = cd[J];
        char buf[200];
        std::snprintf(buf, sizeof buf, "You are trying to assemble values in to K[%lld, %lld], but K[%lld, %lld] is missing in the sparsity pattern.",
                      (long long)row, (long long)col, (long long)row, (long long)col);
        return set_error(h, FE_ERR_PATTERN_MISSING, buf, cell, 0, row, col);
    }
    h->last = fe_error_info{};
    return FE_OK;
}

// Shared-memory caps of the kernel's layout from a plan's largest tile of each kind
void set_plan_caps(KernelArgs& A, const Plan& pl) {
    A.rec_cap = std::max(pl.max_rec, 64);
    A.node_cap = std::max(pl.max_nodes, 1);
    A.stage_cap = std::max(pl.max_stage, 2);
    A.out_cap = std::max(pl.max_out, 2);
}

// The kernel compiled for this problem's subdomains, physics and precision (nullptr: none);
// ea_only picks the gather-only form (every subdomain two-phase)
const KernelEntry* find_kernel(const HostProblem& hp, int phys, bool fp64, bool ea_only = false) {
    for (const KernelEntry& e : registry()) {
        if (e.phys != phys || e.fp64 != (int)fp64 || e.ea_only != (int)ea_only) continue;
        bool ok = true;
        for (int s = 0; s < MAX_SUB; ++s) {
            if (s < (int)hp.subs.size()) {
                if (e.kind[s] != hp.subs[s].kind || e.nq[s] != hp.subs[s].nq) ok = false;
            } else if (e.kind[s] >= 0) {
                ok = false;
            }
        }
        if (ok) return &e;
    }
    return nullptr;
}

void device_attributes(fe_handle* h) {
    if (h->max_smem) return;
    cudaDeviceGetAttribute(&h->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
    cudaDeviceGetAttribute(&h->n_sm, cudaDevAttrMultiProcessorCount, h->device);
}

// Dynamic shared memory of one CTA of kernel ke with A's caps; sets A.groups (cell-table
// buffers: one per lane group, fewer when the tables are large) and A.chunk_bytes.
// Shape-table bytes the tile kernel copies to shared memory: none when every subdomain is in
// the two-phase form (no geometry in the tiles)
int tile_shape_bytes(const fe_handle* h, const KernelArgs& A, bool fp64) {
    for (int s = 0; s < A.n_sub; ++s)
        if (!A.ea[s]) return h->shape_bytes[fp64 ? 1 : 0];
    return 0;
}

int tile_smem(fe_handle* h, const KernelEntry* ke, KernelArgs& A, bool fp64) {
    if (ke->ea_only) A.node_cap = 0;  // no coordinates in the gather-only form
    const int fixed = smem_layout(A, tile_shape_bytes(h, A, fp64), fp64 ? 8 : 4).chunk;
    device_attributes(h);
    const int budget = h->max_smem - 1024;  // static shared (mbarriers) headroom
    int tb = 0;
    for (int s = 0; s < MAX_SUB; ++s) {
        A.groups[s] = 0;
        if (ke->kind[s] < 0) continue;
        if (s < A.n_sub && A.ea[s]) {  // two-phase: lane groups without cell tables
            A.groups[s] = ke->groups[s];
            continue;
        }
        const int room = (budget - fixed) / std::max(ke->table_bytes[s], 1);
        A.groups[s] = std::max(1, std::min(ke->groups[s], room));
        tb = std::max(tb, ke->table_bytes[s] * A.groups[s]);
    }
    A.chunk_bytes = tb;
    return fixed + chunk_region_bytes(A);
}

// Upload h->plan's records (replacing the previous plan's device copy) and set the caps the
// kernel's shared-memory layout is sized from. The host copy of the records is released.
cudaError_t install_plan(fe_handle* h) {
    Plan& pl = h->plan;
    KernelArgs& A = h->base;
    char* rec = nullptr;
    int64_t* roff = nullptr;
    cudaError_t e = h->upload(&rec, (const char*)pl.rec.data(), pl.rec.size());
    if (e == cudaSuccess) e = h->upload(&roff, pl.rec_off.data(), pl.rec_off.size());
    if (e != cudaSuccess) {
        if (rec) h->release(rec);
        return e;
    }
    if (A.rec) h->release((void*)A.rec);
    if (A.rec_off) h->release((void*)A.rec_off);
    A.rec = rec;
    A.rec_off = roff;
    decltype(pl.rec)().swap(pl.rec);  // the device copy is the one in use
    A.n_tiles = (int32_t)pl.n_tiles;
    set_plan_caps(A, pl);
    return cudaSuccess;
}

// The dynamic shared-memory limit is a per-kernel, process-wide attribute: raise it when a
// launch needs more than any earlier one (never lower it under another handle's launches).
cudaError_t ensure_smem_attribute(const void* fn, int smem) {
    static std::mutex mu;
    static std::vector<std::pair<const void*, int>> set;
    std::lock_guard<std::mutex> lock(mu);
    for (auto& x : set)
        if (x.first == fn) {
            if (x.second >= smem) return cudaSuccess;
            const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e == cudaSuccess) x.second = smem;
            return e;
        }
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) set.push_back({fn, smem});
    return e;
}

// Device status to "no error": keys all ones, counters zero (memsets, so it can be captured)
cudaError_t status_reset(fe_handle* h, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(h->status_d, 0xFF, 2 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(&h->status_d->flagged, 0, 2 * sizeof(unsigned int), st);
    return e;
}

// Two CTAs per SM (three for the gather-only form) hide each other's record and coordinate
// waits. The plan's tiles are sized from the staging capacity, but its largest record and
// node list follow from the mesh (on a lattice-aligned mesh more tiles snap to their upper
// size), so kernel ke may land just past that line. Then re-plan with a slightly smaller capacity, once per kernel; a kernel
// far past the line (more than a tenth) keeps the plan: smaller tiles would cost more visits
// than the second CTA wins. Returns FE_OK or a CUDA failure of the upload.
int fit_plan(fe_handle* h, const KernelEntry* ke, cudaStream_t st, unsigned ea_mask) {
    h->fitted_fn = ke->fn;
    h->fitted_mask = ea_mask;
    auto with_form = [&](KernelArgs& X) {
        for (int s = 0; s < MAX_SUB; ++s) X.ea[s] = (ea_mask >> s) & 1u ? (const void*)&h->base : nullptr;  // markers only
    };
    KernelArgs A = h->base;
    with_form(A);
    const int smem = tile_smem(h, ke, A, false);
    if (smem > h->max_smem - 1024 || ensure_smem_attribute(ke->fn, smem) != cudaSuccess) return FE_OK;
    int n = 0, n0 = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ke->fn, THREADS, smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n0, ke->fn, THREADS, 0) != cudaSuccess)
        return FE_OK;
    const int want = std::min(n0, ke->ea_only ? 3 : 2);
    if (n >= want) return FE_OK;
    int per_sm = 0, reserved = 0;
    cudaFuncAttributes fa{};
    cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, h->device);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, h->device);
    cudaFuncGetAttributes(&fa, ke->fn);
    const int room = per_sm / want - reserved - (int)fa.sharedSizeBytes;
    int over = smem - room, cur = smem;
    if (over <= 0 || over > smem / 10) return FE_OK;
    int cap = h->stage_cap;
    for (int k = 0; k < 3; ++k) {
        cap = std::min(cap - 256, (int)(cap * (1.0 - (double)over / cur)) & ~255);
        if (cap < 2048) return FE_OK;
        PlanOptions opt;
        opt.stage_cap = cap;
        Plan pl;
        Error err;
        if (build_plan(h->hp, opt, pl, err) != FE_OK || check_plan(h->hp, pl, err) != FE_OK) return FE_OK;
        KernelArgs B = h->base;
        with_form(B);
        set_plan_caps(B, pl);
        cur = tile_smem(h, ke, B, false);
        over = cur - room;
        if (over > 0) continue;
        int m = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, ke->fn, THREADS, cur) != cudaSuccess || m < want) return FE_OK;
        // the records in use are released: let assemblies still reading them finish
        if (h->pending) {
            const int rc = fe_sync(h);
            (void)rc;
        }
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(h, e, "re-plan: stream synchronize");
        h->plan = std::move(pl);
        if ((e = install_plan(h)) != cudaSuccess) return cuda_fail(h, e, "re-plan: upload plan");
        h->stage_cap = cap;
        return FE_OK;
    }
    return FE_OK;
}

// One element_kernel launch over the cells of subdomain s: into the two-phase scratch, or
// (to_caller) into the caller's element arrays
int launch_elements(fe_handle* h, const KernelArgs& A, int s, int phys, bool fp64, cudaStream_t st, const EaOut& eo,
                    bool to_caller) {
    cudaError_t e;
    const SubDev& sd = A.sub[s];
    const ElemEntry* ee = find_elem(sd.kind, sd.nq, phys, fp64);
    if (!ee) return set_error(h, FE_ERR_UNSUPPORTED, "no element kernel compiled for this element / physics");
    // the tensor-core form (128 threads, one cell at a time per CTA) where one exists
    const bool tc = !to_caller && ee->fn_tc && A.tensor;
    const void* fn = tc ? ee->fn_tc : to_caller ? ee->fn_out : ee->fn;
    const int threads = tc ? 128 : THREADS;
    const int pi = fp64 ? 1 : 0;
    const int o1 = h->shape_off1[pi], o2 = h->shape_off2[pi], sb = h->shape_bytes[pi];
    const int off = s == 0 ? 0 : (s == 1 ? o1 : o2);
    const int end = s + 1 < A.n_sub ? (s == 0 ? o1 : o2) : sb;
    int sub_bytes = end - off;
    device_attributes(h);
    const int esmem = tc ? tc_layout(sub_bytes).bytes : ((sub_bytes + 15) & ~15) + ee->groups * ee->group_bytes;
    if (esmem > h->max_smem - 1024) return set_error(h, FE_ERR_UNSUPPORTED, "element tables do not fit in shared memory");
    if ((e = ensure_smem_attribute(fn, esmem)) != cudaSuccess) return cuda_fail(h, e, "cudaFuncSetAttribute");
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, esmem)) != cudaSuccess)
        return cuda_fail(h, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    const int64_t cells_per_cta = tc ? 1 : ee->groups;
    const int64_t need = (sd.n_cells + cells_per_cta - 1) / cells_per_cta;
    // the tensor-core form: three CTAs per SM by its launch bounds (three TMEM allocations of
    // 128 columns fit an SM's 512; a CTA that does not fit waits for one to finish)
    if (tc) per_sm = std::max(per_sm, 3);
    const int64_t egrid = std::min<int64_t>(need, (int64_t)std::max(per_sm, 1) * std::max(h->n_sm, 1));
    if (egrid <= 0) return FE_OK;
    SubDev sdv = sd;
    const void* eshp = (const char*)(fp64 ? (const void*)h->shape_d : (const void*)h->shape_f) + off;
    EaOut eov = eo;
    KernelArgs Av = A;
    void* eargs[] = {(void*)&Av, (void*)&sdv, (void*)&eshp, (void*)&sub_bytes, (void*)&eov};
    e = cudaLaunchKernel(fn, dim3((unsigned)egrid), dim3(threads), eargs, (size_t)esmem, st);
    if (e != cudaSuccess) return cuda_fail(h, e, "element kernel launch");
    return FE_OK;
}

// Shared-memory sizing, status reset and the launch of one assembly: persistent CTAs, as
// many as fit on the device at once (never more than there are tiles).
int launch_assembly(fe_handle* h, const KernelEntry* ke, KernelArgs& A, bool fp64, cudaStream_t st,
                    std::pair<cudaEvent_t, cudaEvent_t>* ev) {
    cudaError_t e;
    const int pi = fp64 ? 1 : 0;
    const int smem = tile_smem(h, ke, A, fp64);
    const int n_sm = h->n_sm;
    if (smem > h->max_smem - 1024) return set_error(h, FE_ERR_UNSUPPORTED, "tile does not fit in shared memory");
    if ((e = ensure_smem_attribute(ke->fn, smem)) != cudaSuccess) return cuda_fail(h, e, "cudaFuncSetAttribute");
    if (ke->fn != h->occ_fn || smem != h->occ_smem) {
        int per_sm = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ke->fn, THREADS, smem)) != cudaSuccess)
            return cuda_fail(h, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        h->occ_fn = ke->fn;
        h->occ_smem = smem;
        h->occ_per_sm = std::max(per_sm, 1);
    }
    const int64_t grid = std::min<int64_t>(A.n_tiles, (int64_t)h->occ_per_sm * std::max(n_sm, 1));
    if (!h->capturing && !h->accumulate_status && (e = status_reset(h, st)) != cudaSuccess) return cuda_fail(h, e, "status reset");
    A.status = h->status_d;
    const void* shp = fp64 ? (const void*)h->shape_d : (const void*)h->shape_f;
    int sb = h->shape_bytes[pi], o1 = h->shape_off1[pi], o2 = h->shape_off2[pi];
    int tsb = tile_shape_bytes(h, A, fp64);
    void* args[] = {(void*)&A, (void*)&shp, (void*)&tsb, (void*)&o1, (void*)&o2};
    if (ev) cudaEventRecord(ev->first, st);
    // two-phase form: the element matrices of those subdomains first
    for (int s = 0; s < A.n_sub; ++s) {
        if (!A.ea[s]) continue;
        EaOut eo{const_cast<void*>(A.ea[s]), nullptr, {A.ea_stride[s], 0, 0}, {0, 0}};
        const int rc = launch_elements(h, A, s, ke->phys, fp64, st, eo, false);
        if (rc != FE_OK) return rc;
    }
    if (grid > 0) {
        e = cudaLaunchKernel(ke->fn, dim3((unsigned)grid), dim3(THREADS), args, (size_t)smem, st);
        if (e != cudaSuccess) return cuda_fail(h, e, "tile kernel launch");
    }
    if (ev) cudaEventRecord(ev->second, st);
    return FE_OK;
}

}  // namespace

// Facet sets of a handle (fe_facet_set_create / fe_assemble_facet_load)
struct fe_facet_set {
    fe_handle* h = nullptr;
    FacetArgs args{};
    int64_t n_rows = 0;
    int64_t *rptr = nullptr, *rows = nullptr, *epos = nullptr;
    DevStatus* status = nullptr;
    DevStatus* status_h = nullptr;
    DeviceBuffers mem;
    template <typename T>
    cudaError_t upload(T** p, const T* src, size_t count) {
        return mem.upload(p, src, count);
    }
    ~fe_facet_set() {
        if (status_h) cudaFreeHost(status_h);
    }
};

// Reference tangents u, v of a facet: the weighted normal is (J u) x (J v) in 3D and
// ((J u)_2, -(J u)_1) in 2D, Ferrite's weighted_normal per reference shape and facet
// (src/FEValues/facet_integrals.jl: quadrilateral 122-129, triangle 154-160, hexahedron
// 190-199, tetrahedron 226-234, prism 264-273). Returns false for an unknown facet.
bool facet_tangent_table(int32_t cell_type, int32_t facet, double* uv) {
    for (int k = 0; k < 6; ++k) uv[k] = 0.0;
    double* u = uv;
    double* v = uv + 3;
    switch (cell_type) {
        case FE_QUADRILATERAL: {
            static const double T[4][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}};
            if (facet < 1 || facet > 4) return false;
            u[0] = T[facet - 1][0];
            u[1] = T[facet - 1][1];
            return true;
        }
        case FE_TRIANGLE: {
            static const double T[3][2] = {{-1, 1}, {0, -1}, {1, 0}};
            if (facet < 1 || facet > 3) return false;
            u[0] = T[facet - 1][0];
            u[1] = T[facet - 1][1];
            return true;
        }
        case FE_HEXAHEDRON: {
            static const int T[6][2] = {{1, 0}, {0, 2}, {1, 2}, {2, 0}, {2, 1}, {0, 1}};
            if (facet < 1 || facet > 6) return false;
            u[T[facet - 1][0]] = 1;
            v[T[facet - 1][1]] = 1;
            return true;
        }
        case FE_TETRAHEDRON: {
            static const double T[4][6] = {{0, 1, 0, 1, 0, 0}, {1, 0, 0, 0, 0, 1}, {1, 0, -1, 0, 1, -1}, {0, 0, 1, 0, 1, 0}};
            if (facet < 1 || facet > 4) return false;
            for (int k = 0; k < 6; ++k) uv[k] = T[facet - 1][k];
            return true;
        }
        case FE_WEDGE: {
            static const double T[5][6] = {{0, 1, 0, 1, 0, 0}, {1, 0, 0, 0, 0, 1}, {0, 0, 1, 0, 1, 0}, {-1, 1, 0, 0, 0, 1}, {1, 0, 0, 0, 1, 0}};
            if (facet < 1 || facet > 5) return false;
            for (int k = 0; k < 6; ++k) uv[k] = T[facet - 1][k];
            return true;
        }
    }
    return false;
}

// Dirichlet constraints of a handle (fe_dirichlet_create / fe_apply)
struct fe_dirichlet {
    fe_handle* h = nullptr;
    int64_t n = 0, np = 0, n_rows = 0, n_zero = 0;
    int64_t* pd0 = nullptr;    // [np] prescribed dofs, 0-based ascending
    int64_t* diag = nullptr;   // [n] nzval index of K[i, i], -1 if the pattern has none
    int64_t* pdiag = nullptr;  // [np] nzval index of K[d, d]
    int64_t* zero = nullptr;   // [n_zero] entries of the prescribed columns and rows
    int64_t* rptr = nullptr;   // [n_rows + 1] per row with prescribed-column entries:
    int64_t* rows = nullptr;   // [n_rows]     the row,
    int64_t* epos = nullptr;   //              its entries' nzval indices and
    int32_t* epi = nullptr;    //              prescribed-dof numbers, in prescribed order
    double* g = nullptr;       // [np] inhomogeneities of the current call
    double* part = nullptr;    // [DIAG_BLOCKS] meandiag partial sums
    double* m = nullptr;       // meandiag
    DeviceBuffers mem;
    template <typename T>
    cudaError_t upload(T** p, const T* src, size_t count) {
        return mem.upload(p, src, count);
    }
};

// Element-matrix operator of a handle (fe_element_operator_create / fe_element_matvec)
struct fe_element_operator {
    fe_handle* h = nullptr;
    int fp64 = 0;
    bool rows = false;  // a cell's matrix is one block (cell stride != 1): a warp per cell
    int64_t ks[3] = {0, 0, 0};
    int64_t ndofs = 0;
    struct Sub {
        int32_t n = 0;              // dofs per cell
        int64_t n_cells = 0, off = 0;  // cells, first scratch value
        int32_t* cells = nullptr;   // [n_cells] 0-based cell ids
        int32_t* dofs = nullptr;    // 0-based dofs, [n][n_cells] (rows: [n_cells][n])
    };
    std::vector<Sub> subs;
    int64_t* ptr = nullptr;  // [ndofs + 1] incidences of each dof
    int32_t* inc = nullptr;  //   their scratch positions, in ascending cell order
    void* ye = nullptr;      // scratch: per subdomain [n][n_cells] element products
    DeviceBuffers mem;
    template <typename T>
    cudaError_t upload(T** p, const T* src, size_t count) {
        return mem.upload(p, src, count);
    }
};

namespace {

// the vector form of element_products_rows: J contiguous, every row start 16-byte aligned
template <typename T>
bool rows_vectorizable(int n, const T* ke, const int64_t* ks) {
    constexpr int W = Vec16<T>::W;
    return ks[2] == 1 && ks[1] % W == 0 && ks[0] % W == 0 && n % W == 0 && ((uintptr_t)ke & 15u) == 0;
}

template <typename T, int N>
void launch_rows(bool vec, unsigned grid, cudaStream_t st, const T* ke, const int64_t* ks, const int32_t* cells,
                 const int32_t* dofs, int64_t n_cells, const double* u, T* ye) {
    if constexpr (N % Vec16<T>::W == 0) {
        if (vec) {
            element_products_rows<T, N, true><<<grid, 256, 0, st>>>(ke, ks[0], ks[1], ks[2], cells, dofs, n_cells, u, ye);
            return;
        }
    }
    element_products_rows<T, N, false><<<grid, 256, 0, st>>>(ke, ks[0], ks[1], ks[2], cells, dofs, n_cells, u, ye);
}

template <typename T>
cudaError_t launch_products(int n, bool rows, unsigned grid, cudaStream_t st, const T* ke, const int64_t* ks,
                            const int32_t* cells, const int32_t* dofs, int64_t n_cells, const double* u, T* ye) {
    const bool vec = rows && rows_vectorizable(n, ke, ks);
#define FE_PRODUCTS(N)                                                                                          \
    case N:                                                                                                     \
        if (rows)                                                                                               \
            launch_rows<T, N>(vec, grid, st, ke, ks, cells, dofs, n_cells, u, ye);                              \
        else                                                                                                    \
            element_products<T, N, products_split<T>(N)>                                                        \
                <<<grid, 128, 0, st>>>(ke, ks[0], ks[1], ks[2], cells, dofs, n_cells, u, ye);                   \
        break;
    switch (n) {
        FE_PRODUCTS(3)
        FE_PRODUCTS(4)
        FE_PRODUCTS(6)
        FE_PRODUCTS(8)
        FE_PRODUCTS(9)
        FE_PRODUCTS(12)
        FE_PRODUCTS(18)
        FE_PRODUCTS(24)
        FE_PRODUCTS(27)
        FE_PRODUCTS(81)
        default:
            return cudaErrorInvalidValue;
    }
#undef FE_PRODUCTS
    return cudaGetLastError();
}

bool matvec_supported(int n) {
    return n == 3 || n == 4 || n == 6 || n == 8 || n == 9 || n == 12 || n == 18 || n == 24 || n == 27 || n == 81;
}

}  // namespace

extern "C" {

int fe_abi_version(void) { return FE_ABI_VERSION; }

int fe_create(const fe_grid_desc* grid, int32_t n_subdomains, const fe_subdomain_desc* subdomains, const fe_dof_desc* dofs,
              const fe_csc_desc* pattern, fe_handle** out) {
    if (!out) return FE_ERR_ARG;
    *out = nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    // A device-resident pattern (fe_sparsity_pattern_device, or a CuSparseMatrixCSC's colPtr /
    // rowVal): with both arrays in device memory only colptr comes to the host, and the
    // pattern check and the rank tables (the element -> nzval index map) are built on the
    // device; with one of them on the host, both are read on the host.
    std::vector<int64_t> cp_host, rv_host;
    fe_csc_desc pattern_host{};
    const int64_t *cp_dev = nullptr, *rv_dev = nullptr;
    if (pattern && pattern->n > 0 && pattern->nnz >= 0 && pattern->colptr && pattern->rowval &&
        (is_device_ptr(pattern->colptr) || is_device_ptr(pattern->rowval))) {
        const bool both = is_device_ptr(pattern->colptr) && is_device_ptr(pattern->rowval);
        cp_host.resize((size_t)pattern->n + 1);
        if (!both) rv_host.resize((size_t)pattern->nnz);
        cudaError_t ce = cudaMemcpy(cp_host.data(), pattern->colptr, cp_host.size() * 8, cudaMemcpyDefault);
        if (ce == cudaSuccess && pattern->nnz > 0 && !both)
            ce = cudaMemcpy(rv_host.data(), pattern->rowval, rv_host.size() * 8, cudaMemcpyDefault);
        if (ce != cudaSuccess) {
            g_create_error = fe_error_info{};
            g_create_error.code = FE_ERR_CUDA;
            std::snprintf(g_create_error.message, sizeof(g_create_error.message), "copy of the device pattern: %s",
                          cudaGetErrorString(ce));
            return FE_ERR_CUDA;
        }
        if (both) {
            cp_dev = pattern->colptr;
            rv_dev = pattern->rowval;
        }
        pattern_host = fe_csc_desc{pattern->n, pattern->nnz, cp_host.data(), both ? nullptr : rv_host.data()};
        pattern = &pattern_host;
    }
    fe_handle* h = new (std::nothrow) fe_handle();
    if (!h) return FE_ERR_OOM;
    Error err;
    CreateInput in{grid, n_subdomains, subdomains, dofs, pattern};
    in.device_pattern = rv_dev != nullptr;
    int rc = build_problem(in, h->hp, err);
    if (rc == FE_OK && in.device_pattern) rc = device_index_map(h->hp, cp_dev, rv_dev, err);
    if (rc == FE_OK) {
        PlanOptions opt;
        if (const char* s = std::getenv("FE_GB300_STAGE_CAP")) opt.stage_cap = std::atoi(s);
        rc = build_plan(h->hp, opt, h->plan, err);
        if (rc == FE_OK) rc = check_plan(h->hp, h->plan, err);
        h->stage_cap = opt.stage_cap;
    }
    if (rc != FE_OK) {
        g_create_error = fe_error_info{};
        g_create_error.code = rc;
        g_create_error.cell = err.cell;
        g_create_error.row = err.row;
        g_create_error.col = err.col;
        std::snprintf(g_create_error.message, sizeof(g_create_error.message), "%s", err.msg.c_str());
        delete h;
        return rc;
    }
    const HostProblem& hp = h->hp;
    const Plan& pl = h->plan;
    cudaError_t e = cudaGetDevice(&h->device);
#define CK(x)                                   \
    do {                                        \
        e = (x);                                \
        if (e != cudaSuccess) {                 \
            int c_ = cuda_fail(h, e, #x);       \
            g_create_error = h->last;           \
            delete h;                           \
            return c_;                          \
        }                                       \
    } while (0)
    CK(e);
    KernelArgs& A = h->base;
    A.nc = hp.nc;
    A.dim = hp.dim;
    A.n_sub = (int32_t)hp.subs.size();
    // node coordinates: FP64 [n][dim], and 24 bytes per node for the gathers: float hi
    // (x, y, z) then float lo, or FP64 (x, y, z)
    {
        double* xd;
        CK(h->upload(&xd, hp.nodes.data(), hp.nodes.size()));
        A.xd = xd;
        std::vector<float> x6((size_t)hp.n_nodes * 6, 0.f);
        std::vector<double> x3((size_t)hp.n_nodes * 3, 0.0);
        for (int64_t n = 0; n < hp.n_nodes; ++n)
            for (int x = 0; x < hp.dim; ++x) {
                const double v = hp.nodes[n * hp.dim + x];
                const float hi = (float)v;
                x6[n * 6 + x] = hi;
                x6[n * 6 + 3 + x] = (float)(v - (double)hi);
                x3[n * 3 + x] = v;
            }
        float* xf6;
        double* xd3;
        CK(h->upload(&xf6, x6.data(), x6.size()));
        CK(h->upload(&xd3, x3.data(), x3.size()));
        A.xf6 = xf6;
        A.xd3 = xd3;
    }
    // subdomains
    std::vector<float> shf;
    std::vector<double> shd;
    int offs_f[MAX_SUB] = {0, 0, 0}, offs_d[MAX_SUB] = {0, 0, 0};
    for (size_t s = 0; s < hp.subs.size(); ++s) {
        const HostSub& hs = hp.subs[s];
        SubDev& sd = A.sub[s];
        sd.kind = hs.kind; sd.nb = hs.nb; sd.ng = hs.ng; sd.nq = hs.nq; sd.dim = hs.dim; sd.nc = hs.nc;
        sd.n_cells = hs.n_cells;
        int32_t *cid, *ents, *cconn;
        CK(h->upload(&cid, hs.cellid.data(), hs.cellid.size()));
        CK(h->upload(&ents, hs.ents.data(), hs.ents.size()));
        CK(h->upload(&cconn, hs.conn.data(), hs.conn.size()));
        sd.cellid = cid; sd.ents = ents; sd.conn = cconn;
        // reference tables: one record per quadrature point (dM, dN, N, w; layout shape_q)
        auto push_records = [&](auto& vec) {
            using T = typename std::remove_reference<decltype(vec)>::type::value_type;
            const ShapeQ L = shape_q(hs.nb, hs.ng, hs.dim, (int)sizeof(T));
            const size_t start = vec.size();
            vec.resize(start + (size_t)hs.nq * L.qs, (T)0);
            for (int q = 0; q < hs.nq; ++q) {
                T* r = vec.data() + start + (size_t)q * L.qs;
                for (int t = 0; t < hs.ng * hs.dim; ++t) r[L.dm + t] = (T)hs.dM[(size_t)q * hs.ng * hs.dim + t];
                for (int t = 0; t < hs.nb * hs.dim; ++t) r[L.dn + t] = (T)hs.dN[(size_t)q * hs.nb * hs.dim + t];
                for (int t = 0; t < hs.nb; ++t) r[L.n + t] = (T)hs.N[(size_t)q * hs.nb + t];
                r[L.w] = (T)hs.w[q];
                r[L.w + 1] = (T)std::sqrt(hs.w[q]);
            }
        };
        offs_f[s] = (int)(shf.size() * sizeof(float));
        offs_d[s] = (int)(shd.size() * sizeof(double));
        push_records(shf);
        push_records(shd);
        float *wf, *Nf, *dNf, *dMf;
        double *wd, *Nd, *dNd, *dMd;
        std::vector<float> tmp;
        auto upf = [&](float** p, const std::vector<double>& v) {
            tmp.assign(v.begin(), v.end());
            return h->upload(p, tmp.data(), tmp.size());
        };
        CK(upf(&wf, hs.w)); CK(upf(&Nf, hs.N)); CK(upf(&dNf, hs.dN)); CK(upf(&dMf, hs.dM));
        CK(h->upload(&wd, hs.w.data(), hs.w.size()));
        CK(h->upload(&Nd, hs.N.data(), hs.N.size()));
        CK(h->upload(&dNd, hs.dN.data(), hs.dN.size()));
        CK(h->upload(&dMd, hs.dM.data(), hs.dM.size()));
        sd.w_f = wf; sd.N_f = Nf; sd.dN_f = dNf; sd.dM_f = dMf;
        sd.w_d = wd; sd.N_d = Nd; sd.dN_d = dNd; sd.dM_d = dMd;
    }
    CK(h->upload(&h->shape_f, shf.data(), shf.size()));
    CK(h->upload(&h->shape_d, shd.data(), shd.size()));
    h->shape_bytes[0] = (int)(shf.size() * sizeof(float));
    h->shape_bytes[1] = (int)(shd.size() * sizeof(double));
    h->shape_off1[0] = offs_f[1]; h->shape_off2[0] = offs_f[2];
    h->shape_off1[1] = offs_d[1]; h->shape_off2[1] = offs_d[2];
    // tile records
    A.bs = (hp.nc * hp.nc + 1) & ~1;
    if (pl.n_tiles >= (int64_t)INT32_MAX) {
        set_error(h, FE_ERR_UNSUPPORTED, "too many tiles");
        g_create_error = h->last;
        delete h;
        return FE_ERR_UNSUPPORTED;
    }
    h->plan_pinned = std::getenv("FE_GB300_STAGE_CAP") != nullptr;
    CK(install_plan(h));
    CK(h->alloc(&h->status_d, 1));
    CK(cudaMallocHost((void**)&h->status_h, sizeof(DevStatus)));
#undef CK
    h->create_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = h;
    return FE_OK;
}

// digest of a plan: FNV-1a 64 of each tile record (in parallel), then of those in tile order
static uint32_t plan_digest(const Plan& pl) {
    constexpr uint64_t basis = 1469598103934665603ull, prime = 1099511628211ull;
    std::vector<uint64_t> th((size_t)pl.n_tiles);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < pl.n_tiles; ++t) {
        uint64_t h = basis;
        for (int64_t b = pl.rec_off[t]; b < pl.rec_off[t + 1]; ++b) {
            h ^= pl.rec[(size_t)b];
            h *= prime;
        }
        th[(size_t)t] = h;
    }
    uint64_t h = basis;
    for (const uint64_t v : th)
        for (int k = 0; k < 8; ++k) {
            h ^= (v >> (8 * k)) & 0xFFu;
            h *= prime;
        }
    return (uint32_t)(h ^ (h >> 32));
}

int fe_plan_dry_run(const fe_grid_desc* grid, int32_t n_subdomains, const fe_subdomain_desc* subdomains,
                    const fe_dof_desc* dofs, const fe_csc_desc* pattern, fe_info* out) {
    if (!out) return FE_ERR_ARG;
    const auto t0 = std::chrono::steady_clock::now();
    HostProblem hp;
    Plan pl;
    Error err;
    CreateInput in{grid, n_subdomains, subdomains, dofs, pattern};
    int rc = build_problem(in, hp, err);
    PlanOptions opt;
    if (const char* s = std::getenv("FE_GB300_STAGE_CAP")) opt.stage_cap = std::atoi(s);
    if (rc == FE_OK) rc = build_plan(hp, opt, pl, err);
    if (rc == FE_OK) rc = check_plan(hp, pl, err);
    if (rc != FE_OK) {
        g_create_error = fe_error_info{};
        g_create_error.code = rc;
        g_create_error.cell = err.cell;
        g_create_error.row = err.row;
        g_create_error.col = err.col;
        std::snprintf(g_create_error.message, sizeof(g_create_error.message), "%s", err.msg.c_str());
        return rc;
    }
    *out = fe_info{};
    out->n_cells = hp.n_cells;
    out->ndofs = hp.ndofs;
    out->nnz = hp.nnz;
    out->n_tiles = pl.n_tiles;
    out->n_cell_visits = pl.visits;
    out->n_items = pl.items;
    out->max_record_bytes = pl.max_rec;
    out->max_tile_nodes = pl.max_nodes;
    out->max_stage_values = pl.max_stage;
    out->max_out_doubles = pl.max_out;
    out->stage_cap = opt.stage_cap;
    out->plan_checksum = plan_digest(pl);
    out->create_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return FE_OK;
}

void fe_destroy(fe_handle* h) {
    if (!h) return;
    if (h->pending) cudaStreamSynchronize(h->last_stream);
    delete h;
}

int fe_sync(fe_handle* h) {
    if (!h) return FE_ERR_ARG;
    if (!h->pending) return h->last.code;
    cudaError_t e = cudaStreamSynchronize(h->last_stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamSynchronize");
    return finish_status(h);
}

// fe_assemble, or with eo the element assembly of fe_assemble_elements (no global matrix:
// every cell's Ke and fe into the caller's device arrays)
static int assemble_common(fe_handle* h, const fe_assemble_params* p, double* nzval, double* f, const EaOut* eo) {
    if (!h || !p) return FE_ERR_ARG;
    const HostProblem& hp = h->hp;
    const int nc = hp.nc;
    int phys = 0;
    switch (p->physics) {
        case FE_HEAT:
            if (nc != 1) return set_error(h, FE_ERR_ARG, "FE_HEAT needs a scalar field");
            phys = PHYS_HEAT;
            break;
        case FE_LINEAR_ELASTIC:
            if (nc != hp.dim) return set_error(h, FE_ERR_ARG, "FE_LINEAR_ELASTIC needs a dim-component field");
            phys = PHYS_ELASTIC;
            break;
        case FE_NEO_HOOKE:
            if (nc != 3 || hp.dim != 3) return set_error(h, FE_ERR_ARG, "FE_NEO_HOOKE needs a 3-component field in 3D");
            if (!p->u) return set_error(h, FE_ERR_ARG, "FE_NEO_HOOKE needs u");
            phys = PHYS_NEO;
            break;
        default:
            return set_error(h, FE_ERR_ARG, "unknown physics");
    }
    if (p->precision != FE_PREC_MIXED && p->precision != FE_PREC_FP64) return set_error(h, FE_ERR_ARG, "unknown precision");
    const bool fp64 = p->precision == FE_PREC_FP64;
    const bool do_k = !(p->flags & FE_NO_K), do_f = !(p->flags & FE_NO_F);
    if (eo) {
        if (do_k && !eo->ke) return set_error(h, FE_ERR_ARG, "ke is NULL");
        if (do_f && !eo->fe) return set_error(h, FE_ERR_ARG, "fe is NULL");
        if ((do_k && !is_device_ptr(eo->ke)) || (do_f && !is_device_ptr(eo->fe)))
            return set_error(h, FE_ERR_ARG, "element arrays must be device memory");
    } else {
        if (do_k && !nzval) return set_error(h, FE_ERR_ARG, "nzval is NULL");
        if (do_f && !f) return set_error(h, FE_ERR_ARG, "f is NULL");
    }
    // two-phase form per subdomain: quadratic elements by default (their geometry would be
    // recomputed in every tile that owns one of their ~27 dof entities)
    // (or the form fe_autotune chose for this physics and precision, when the call names none)
    unsigned ea_mask = 0;
    bool all_ea = true;
    const bool named = (p->flags & (FE_TWO_PHASE | FE_FUSED)) != 0;
    const bool tuned = !named && h->tuned_valid && h->tuned_phys == p->physics && h->tuned_prec == p->precision;
    for (int s = 0; s < (int)hp.subs.size() && !eo; ++s) {
        bool two;
        if (h->force_on) two = (h->force_mask >> s) & 1u;
        else if (tuned) two = (h->tuned_mask >> s) & 1u;
        else two = (p->flags & FE_TWO_PHASE) || (!(p->flags & FE_FUSED) && hp.subs[s].nb > 16);
        if (hp.subs[s].n_cells > 0 && two)
            ea_mask |= 1u << s;
        else if (hp.subs[s].n_cells > 0)
            all_ea = false;
    }
    const KernelEntry* ke = all_ea && ea_mask ? find_kernel(hp, phys, fp64, true) : nullptr;
    if (!ke) ke = find_kernel(hp, phys, fp64);
    if (!ke) return set_error(h, FE_ERR_UNSUPPORTED, "no kernel compiled for this element / quadrature / physics combination");
    if (!eo && !fp64 && !h->capturing && !h->plan_pinned && (h->fitted_fn != ke->fn || h->fitted_mask != ea_mask)) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing((cudaStream_t)p->stream, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
            const int rc = fit_plan(h, ke, (cudaStream_t)p->stream, ea_mask);
            if (rc != FE_OK) return rc;
        }
    }
    if (h->capturing) {
        // inside fe_graph_capture: device buffers only, the capture stream, no host work
        if ((cudaStream_t)p->stream != h->cap_stream) return set_error(h, FE_ERR_STATE, "capture: steps run on the capture stream");
        if (p->flags & FE_PROFILE) return set_error(h, FE_ERR_STATE, "capture: FE_PROFILE is not capturable");
        if ((!eo && ((do_k && !is_device_ptr(nzval)) || (do_f && !is_device_ptr(f)))) || (p->u && !is_device_ptr(p->u)) ||
            (p->cell_scale && !is_device_ptr(p->cell_scale)))
            return set_error(h, FE_ERR_STATE, "capture: nzval, f, u and cell_scale must be device memory");
    } else if (h->pending) {
        // An FE_ASYNC assembly on the same stream with device outputs is still running: keep
        // its status and let this one add to it (fe_sync reports both), without waiting.
        // Anything else waits for it first.
        const bool chain = (cudaStream_t)p->stream == h->last_stream &&
                           (eo || ((!do_k || is_device_ptr(nzval)) && (!do_f || is_device_ptr(f))));
        if (chain) {
            h->accumulate_status = 1;
        } else {
            int rc = fe_sync(h);
            (void)rc;
        }
    }
    cudaStream_t st = (cudaStream_t)p->stream;
    cudaError_t e;
    KernelArgs A = h->base;
    // outputs: device pointers are written in place, page-locked host memory through its
    // mapping (plain stores) unless FE_STAGED_OUTPUT, other host memory is staged
    const bool mapped_out = !eo && !h->capturing && !(p->flags & FE_STAGED_OUTPUT);
    double* nz_map = mapped_out && do_k && !is_device_ptr(nzval) ? (double*)pinned_device_alias(nzval) : nullptr;
    double* f_map = mapped_out && do_f && !is_device_ptr(f) ? (double*)pinned_device_alias(f) : nullptr;
    const bool nz_dev = eo || (do_k && (nz_map || is_device_ptr(nzval)));
    const bool f_dev = eo || (do_f && (f_map || is_device_ptr(f)));
    const bool fill = (p->flags & FE_FILLZERO) != 0;
    if (do_k && !nz_dev) {
        if (!h->nz_stage && (e = h->alloc(&h->nz_stage, hp.nnz)) != cudaSuccess) return cuda_fail(h, e, "alloc nzval");
        if (!fill && (e = cudaMemcpyAsync(h->nz_stage, nzval, hp.nnz * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return cuda_fail(h, e, "copy nzval");
    }
    if (do_f && !f_dev) {
        if (!h->f_stage && (e = h->alloc(&h->f_stage, hp.ndofs)) != cudaSuccess) return cuda_fail(h, e, "alloc f");
        if (!fill && (e = cudaMemcpyAsync(h->f_stage, f, hp.ndofs * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return cuda_fail(h, e, "copy f");
    }
    A.nzval = do_k && !eo ? (nz_map ? nz_map : nz_dev ? nzval : h->nz_stage) : nullptr;
    A.f = do_f && !eo ? (f_map ? f_map : f_dev ? f : h->f_stage) : nullptr;
    A.host_out = nz_map != nullptr;
    A.tensor = (p->flags & FE_NO_TENSOR) ? 0 : 1;
    A.do_k = do_k;
    A.do_f = do_f;
    A.fillzero = fill;
    A.compensated = (p->flags & FE_FP32_SUM) == 0;  // compensated unless plain FP32 sums are asked for
    // element-matrix scratch of the two-phase subdomains
    {
        size_t need = 0;
        int64_t offs[MAX_SUB] = {0, 0, 0};
        const size_t rb = fp64 ? sizeof(double) : sizeof(float);
        for (int s = 0; s < (int)hp.subs.size(); ++s) {
            const HostSub& hs = hp.subs[s];
            A.ea[s] = nullptr;
            A.ea_stride[s] = 0;
            if (!((ea_mask >> s) & 1u)) continue;
            offs[s] = (int64_t)need;
            A.ea_stride[s] = ea_cell_values(hs.nb, hs.nc);
            need += (size_t)hs.n_cells * (size_t)A.ea_stride[s] * rb;
            A.ea[s] = (const void*)1;  // placed below
        }
        if (need > h->ea_bytes) {
            if (h->capturing) return set_error(h, FE_ERR_STATE, "capture: the two-phase scratch grows; assemble once before capturing");
            if (h->ea_buf) h->release(h->ea_buf);
            h->ea_buf = nullptr;
            h->ea_bytes = 0;
            char* b = nullptr;
            if ((e = h->alloc(&b, need)) != cudaSuccess) return cuda_fail(h, e, "alloc element-matrix scratch");
            h->ea_buf = b;
            h->ea_bytes = need;
        }
        for (int s = 0; s < (int)hp.subs.size(); ++s)
            if (A.ea[s]) A.ea[s] = (const char*)h->ea_buf + offs[s];
    }
    // inputs
    Physics& ph = A.phys;
    ph = Physics{};
    ph.kind = p->physics;
    ph.p0 = p->p0;
    ph.p1 = p->p1;
    for (int x = 0; x < 3; ++x) ph.body[x] = p->body[x];
    if (p->physics == FE_LINEAR_ELASTIC) {
        const double E = p->p0, nu = p->p1;
        ph.lam = E * nu / ((1 + nu) * (1 - 2 * nu));
        ph.mu = E / (2 * (1 + nu));
    }
    ph.cond_threshold = p->cond_threshold > 0 ? (float)p->cond_threshold : 64.0f;
    ph.p0_f = (float)ph.p0;
    ph.p1_f = (float)ph.p1;
    ph.lam_f = (float)ph.lam;
    ph.mu_f = (float)ph.mu;
    for (int x = 0; x < 3; ++x) ph.body_f[x] = (float)ph.body[x];
    auto stage_input = [&](const double* src, int64_t n, double** stage, float** stage_f, const double** out_d,
                           const float** out_f) -> int {
        const double* dsrc = src;
        if (!is_device_ptr(src)) {
            if (!*stage && (e = h->alloc(stage, n)) != cudaSuccess) return cuda_fail(h, e, "alloc input");
            if ((e = cudaMemcpyAsync(*stage, src, n * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess)
                return cuda_fail(h, e, "copy input");
            dsrc = *stage;
        }
        *out_d = dsrc;
        if (!fp64) {
            if (!*stage_f && (e = h->alloc(stage_f, n)) != cudaSuccess) return cuda_fail(h, e, "alloc input");
            to_float_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(dsrc, *stage_f, n);
            *out_f = *stage_f;
        }
        return FE_OK;
    };
    if (p->cell_scale) {
        int rc = stage_input(p->cell_scale, hp.n_cells, &h->scale_stage, &h->scale_f, &ph.scale_d, &ph.scale_f);
        if (rc) return rc;
        if (fp64) ph.scale_f = (const float*)ph.scale_d;  // non-null marker; the FP64 kernel reads scale_d
    }
    if (p->physics == FE_NEO_HOOKE) {
        int rc = stage_input(p->u, hp.ndofs, &h->u_stage, &h->u_f, &ph.u_d, &ph.u_f);
        if (rc) return rc;
    }
    std::pair<cudaEvent_t, cudaEvent_t> ev{nullptr, nullptr};
    const bool prof = (p->flags & FE_PROFILE) != 0;
    if (prof) {
        if (!h->prof_pool.empty()) {
            ev = h->prof_pool.back();
            h->prof_pool.pop_back();
        } else if ((e = cudaEventCreate(&ev.first)) != cudaSuccess || (e = cudaEventCreate(&ev.second)) != cudaSuccess) {
            return cuda_fail(h, e, "cudaEventCreate");
        }
    }
    if (eo) {
        // element assembly: status reset, then the element kernels of every subdomain
        if (!h->capturing && !h->accumulate_status && (e = status_reset(h, st)) != cudaSuccess)
            return cuda_fail(h, e, "status reset");
        A.status = h->status_d;
        if (prof) cudaEventRecord(ev.first, st);
        int rc = FE_OK;
        for (int s = 0; s < A.n_sub && rc == FE_OK; ++s) rc = launch_elements(h, A, s, ke->phys, fp64, st, *eo, true);
        if (prof) {
            cudaEventRecord(ev.second, st);
            (rc == FE_OK ? h->prof_events : h->prof_pool).push_back(ev);
        }
        if (rc != FE_OK) return rc;
    } else {
        const int rc = launch_assembly(h, ke, A, fp64, st, prof ? &ev : nullptr);
        if (prof) (rc == FE_OK ? h->prof_events : h->prof_pool).push_back(ev);
        if (rc != FE_OK) return rc;
    }
    if (h->capturing) return FE_OK;  // the capture reads the status once, after its last step
    if ((e = cudaMemcpyAsync(h->status_h, h->status_d, sizeof(DevStatus), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(h, e, "status read");
    if (do_k && !nz_dev && (e = cudaMemcpyAsync(nzval, h->nz_stage, hp.nnz * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(h, e, "copy nzval back");
    if (do_f && !f_dev && (e = cudaMemcpyAsync(f, h->f_stage, hp.ndofs * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(h, e, "copy f back");
    h->last_stream = st;
    h->pending = 1;
    const bool host_out = (do_k && !nz_dev) || (do_f && !f_dev);
    if ((p->flags & FE_ASYNC) && !host_out) return FE_OK;
    return fe_sync(h);
}

int fe_assemble(fe_handle* h, const fe_assemble_params* p, double* nzval, double* f) {
    return assemble_common(h, p, nzval, f, nullptr);
}

int fe_assemble_elements(fe_handle* h, const fe_assemble_params* p, void* ke, void* fe, const fe_element_layout* layout) {
    if (!h || !p || !layout) return FE_ERR_ARG;
    EaOut eo{ke, fe, {layout->ke_stride[0], layout->ke_stride[1], layout->ke_stride[2]},
             {layout->fe_stride[0], layout->fe_stride[1]}};
    return assemble_common(h, p, nullptr, nullptr, &eo);
}

int fe_assemble_adjoint(fe_handle* h, const fe_adjoint_params* p, const double* u, const double* lambda, double* d_rho,
                        double* d_X) {
    if (!h || !p || !u || !lambda || !d_rho) return FE_ERR_ARG;
    const HostProblem& hp = h->hp;
    const int nc = hp.nc, dim = hp.dim;
    int phys = 0;
    if (p->physics == FE_HEAT) {
        if (nc != 1) return set_error(h, FE_ERR_ARG, "FE_HEAT needs a scalar field");
        phys = PHYS_HEAT;
    } else if (p->physics == FE_LINEAR_ELASTIC) {
        if (nc != dim) return set_error(h, FE_ERR_ARG, "FE_LINEAR_ELASTIC needs a dim-component field");
        phys = PHYS_ELASTIC;
    } else {
        return set_error(h, FE_ERR_UNSUPPORTED, "the adjoint supports FE_HEAT and FE_LINEAR_ELASTIC");
    }
    if (p->precision != FE_PREC_MIXED && p->precision != FE_PREC_FP64) return set_error(h, FE_ERR_ARG, "unknown precision");
    const bool fp64 = p->precision == FE_PREC_FP64;
    std::vector<const AdjEntry*> ke(hp.subs.size(), nullptr);
    for (size_t s = 0; s < hp.subs.size(); ++s) {
        for (const AdjEntry& e : adj_registry())
            if (e.kind == hp.subs[s].kind && e.nq == hp.subs[s].nq && e.phys == phys && e.fp64 == (int)fp64) ke[s] = &e;
        if (!ke[s]) return set_error(h, FE_ERR_UNSUPPORTED, "no adjoint kernel for this element / quadrature / physics");
    }
    if (h->pending) fe_sync(h);
    cudaStream_t st = (cudaStream_t)p->stream;
    cudaError_t e;
    // node -> rows (once per handle): rows of subdomain s start at row0[s], cell c, node k
    std::vector<int64_t> row0(hp.subs.size() + 1, 0);
    for (size_t s = 0; s < hp.subs.size(); ++s) row0[s + 1] = row0[s] + hp.subs[s].n_cells * hp.subs[s].ng;
    if (!h->adj_ptr) {
        if (row0.back() >= (int64_t)INT32_MAX) return set_error(h, FE_ERR_UNSUPPORTED, "too many cells for the adjoint");
        std::vector<int64_t> ptr(hp.n_nodes + 1, 0);
        for (const HostSub& hs : hp.subs)
            for (int32_t v : hs.conn) ptr[v + 1]++;
        for (int64_t n = 0; n < hp.n_nodes; ++n) ptr[n + 1] += ptr[n];
        std::vector<int32_t> ids(ptr[hp.n_nodes]);
        std::vector<int64_t> cur(ptr.begin(), ptr.end() - 1);
        for (size_t s = 0; s < hp.subs.size(); ++s) {
            const HostSub& hs = hp.subs[s];
            for (int64_t c = 0; c < hs.n_cells; ++c)
                for (int k = 0; k < hs.ng; ++k) ids[cur[hs.conn[c * hs.ng + k]]++] = (int32_t)(row0[s] + c * hs.ng + k);
        }
        if ((e = h->upload(&h->adj_ptr, ptr.data(), ptr.size())) != cudaSuccess) return cuda_fail(h, e, "adjoint index");
        if ((e = h->upload(&h->adj_row_ids, ids.data(), ids.size())) != cudaSuccess) return cuda_fail(h, e, "adjoint index");
        char* cb = nullptr;
        if ((e = h->alloc(&cb, (size_t)row0.back() * dim * sizeof(double))) != cudaSuccess) return cuda_fail(h, e, "adjoint rows");
        h->adj_contrib = cb;
        h->adj_rows = row0.back();
    }
    AdjArgs A{};
    A.xf6 = h->base.xf6;
    A.xd3 = h->base.xd3;
    // inputs: device pointers are used in place, host pointers staged
    auto stage = [&](const double* src, int64_t n, double** buf) -> const double* {
        if (is_device_ptr(src)) return src;
        if (!*buf && (e = h->alloc(buf, n)) != cudaSuccess) return nullptr;
        if ((e = cudaMemcpyAsync(*buf, src, n * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess) return nullptr;
        return *buf;
    };
    auto to_f = [&](const double* src, int64_t n, float** buf) -> const float* {
        if (!*buf && (e = h->alloc(buf, n)) != cudaSuccess) return nullptr;
        to_float_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(src, *buf, n);
        return *buf;
    };
    if (!(A.u_d = stage(u, hp.ndofs, &h->u_stage)) || !(A.l_d = stage(lambda, hp.ndofs, &h->lam_stage)))
        return cuda_fail(h, e, "adjoint inputs");
    if (!fp64 && (!(A.u_f = to_f(A.u_d, hp.ndofs, &h->u_f)) || !(A.l_f = to_f(A.l_d, hp.ndofs, &h->lam_f))))
        return cuda_fail(h, e, "adjoint inputs");
    if (p->cell_scale) {
        if (!(A.scale_d = stage(p->cell_scale, hp.n_cells, &h->scale_stage))) return cuda_fail(h, e, "cell_scale");
        if (!fp64 && !(A.scale_f = to_f(A.scale_d, hp.n_cells, &h->scale_f))) return cuda_fail(h, e, "cell_scale");
    }
    if (p->dscale && !(A.dscale = stage(p->dscale, hp.n_cells, &h->dscale_stage))) return cuda_fail(h, e, "dscale");
    if (phys == PHYS_HEAT) {
        A.m0 = p->p0;
        A.load[0] = p->p1;
    } else {
        const double E = p->p0, nu = p->p1;
        A.m0 = E * nu / ((1 + nu) * (1 - 2 * nu));
        A.m1 = E / (2 * (1 + nu));
        for (int x = 0; x < 3; ++x) A.load[x] = p->body[x];
    }
    A.m0_f = (float)A.m0;
    A.m1_f = (float)A.m1;
    for (int x = 0; x < 3; ++x) A.load_f[x] = (float)A.load[x];
    // outputs
    const bool rho_dev = is_device_ptr(d_rho), x_dev = d_X && is_device_ptr(d_X);
    double* drho = d_rho;
    if (!rho_dev) {
        if (!h->drho_stage && (e = h->alloc(&h->drho_stage, hp.n_cells)) != cudaSuccess) return cuda_fail(h, e, "alloc d_rho");
        drho = h->drho_stage;
    }
    double* dX = d_X;
    if (d_X && !x_dev) {
        if (!h->dX_stage && (e = h->alloc(&h->dX_stage, hp.n_nodes * dim)) != cudaSuccess) return cuda_fail(h, e, "alloc d_X");
        dX = h->dX_stage;
    }
    if ((e = cudaMemsetAsync(drho, 0, hp.n_cells * sizeof(double), st)) != cudaSuccess) return cuda_fail(h, e, "d_rho");
    A.d_cell = drho;
    A.contrib = h->adj_contrib;
    if ((e = status_reset(h, st)) != cudaSuccess) return cuda_fail(h, e, "status reset");
    A.status = h->status_d;
    int n_sm = 0;
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, h->device);
    for (size_t s = 0; s < hp.subs.size(); ++s) {
        A.row0 = row0[s];
        const SubDev sd = h->base.sub[s];
        const int32_t* conn = sd.conn;
        const void* shp = fp64 ? (const void*)((const char*)h->shape_d + (s ? (s == 1 ? h->shape_off1[1] : h->shape_off2[1]) : 0))
                               : (const void*)((const char*)h->shape_f + (s ? (s == 1 ? h->shape_off1[0] : h->shape_off2[0]) : 0));
        if ((e = cudaFuncSetAttribute(ke[s]->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, ke[s]->smem)) != cudaSuccess)
            return cuda_fail(h, e, "cudaFuncSetAttribute");
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ke[s]->fn, THREADS, ke[s]->smem);
        const int gs = CTA_THREADS / GROUP_LANES[hp.subs[s].kind];
        const int64_t need = (sd.n_cells + gs - 1) / gs;
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)std::max(per_sm, 1) * n_sm * 4));
        void* args[] = {(void*)&A, (void*)&sd, (void*)&conn, (void*)&shp};
        if ((e = cudaLaunchKernel(ke[s]->fn, dim3(grid), dim3(THREADS), args, (size_t)ke[s]->smem, st)) != cudaSuccess)
            return cuda_fail(h, e, "adjoint kernel launch");
    }
    if (d_X) {
        const int64_t n_out = hp.n_nodes * dim;
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n_out + 255) / 256, (int64_t)n_sm * 16));
        const void* contrib = h->adj_contrib;
        int dim32 = dim;
        int64_t nn = hp.n_nodes;
        void* args[] = {(void*)&h->adj_ptr, (void*)&h->adj_row_ids, (void*)&contrib, (void*)&dim32, (void*)&nn, (void*)&dX};
        if ((e = cudaLaunchKernel(adjoint_node_sum_fn(fp64), dim3(grid), dim3(256), args, 0, st)) != cudaSuccess)
            return cuda_fail(h, e, "adjoint node sum launch");
    }
    if ((e = cudaMemcpyAsync(h->status_h, h->status_d, sizeof(DevStatus), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(h, e, "status read");
    if (!rho_dev && (e = cudaMemcpyAsync(d_rho, drho, hp.n_cells * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(h, e, "copy d_rho back");
    if (d_X && !x_dev && (e = cudaMemcpyAsync(d_X, dX, hp.n_nodes * dim * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(h, e, "copy d_X back");
    h->last_stream = st;
    h->pending = 1;
    const bool host_out = !rho_dev || (d_X && !x_dev);
    if ((p->flags & FE_ASYNC) && !host_out) return FE_OK;
    return fe_sync(h);
}

int fe_graph_capture(fe_handle* h, void* stream, int32_t n_steps, const fe_assemble_params* steps, double* const* nzval,
                     double* const* f, int32_t* graph) {
    if (!h || !steps || !nzval || !f || !graph || n_steps < 1) return FE_ERR_ARG;
    if (h->capturing) return set_error(h, FE_ERR_STATE, "a capture is already open");
    cudaStream_t st = (cudaStream_t)stream;
    if (!st) return set_error(h, FE_ERR_ARG, "fe_graph_capture needs a created (non-default) stream");
    for (int32_t k = 0; k < n_steps; ++k) {
        const fe_assemble_params& q = steps[k];
        const bool do_k = !(q.flags & FE_NO_K), do_f = !(q.flags & FE_NO_F);
        if ((do_k && !is_device_ptr(nzval[k])) || (do_f && !is_device_ptr(f[k])) || (q.u && !is_device_ptr(q.u)) ||
            (q.cell_scale && !is_device_ptr(q.cell_scale)))
            return set_error(h, FE_ERR_ARG, "fe_graph_capture: nzval, f, u and cell_scale must be device memory");
    }
    // Run every step once, uncaptured: that allocates the FP32 input copies, sets the kernels'
    // shared-memory attributes and reports element errors before anything is recorded.
    for (int32_t k = 0; k < n_steps; ++k) {
        fe_assemble_params q = steps[k];
        q.stream = st;
        q.flags &= ~(uint32_t)(FE_ASYNC | FE_PROFILE);
        const int rc = fe_assemble(h, &q, nzval[k], f[k]);
        if (rc != FE_OK) return rc;
    }
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamBeginCapture");
    h->capturing = 1;
    h->cap_stream = st;
    int rc = FE_OK;
    if ((e = status_reset(h, st)) != cudaSuccess) rc = cuda_fail(h, e, "status reset");
    for (int32_t k = 0; k < n_steps && rc == FE_OK; ++k) {
        fe_assemble_params q = steps[k];
        q.stream = st;
        q.flags = (q.flags & ~(uint32_t)FE_PROFILE) | FE_ASYNC;
        rc = fe_assemble(h, &q, nzval[k], f[k]);
    }
    if (rc == FE_OK && (e = cudaMemcpyAsync(h->status_h, h->status_d, sizeof(DevStatus), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        rc = cuda_fail(h, e, "status read");
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(st, &g);
    h->capturing = 0;
    if (rc == FE_OK && e != cudaSuccess) rc = cuda_fail(h, e, "cudaStreamEndCapture");
    cudaGraphExec_t x = nullptr;
    if (rc == FE_OK && (e = cudaGraphInstantiate(&x, g, 0)) != cudaSuccess) rc = cuda_fail(h, e, "cudaGraphInstantiate");
    if (rc != FE_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    h->graphs.push_back({g, x});
    *graph = (int32_t)h->graphs.size() - 1;
    return FE_OK;
}

int fe_graph_replay(fe_handle* h, int32_t graph, void* stream, uint32_t flags) {
    if (!h || graph < 0 || graph >= (int32_t)h->graphs.size() || !h->graphs[graph].second) return FE_ERR_ARG;
    if (h->capturing) return set_error(h, FE_ERR_STATE, "replay during a capture");
    if (h->pending) fe_sync(h);
    cudaStream_t st = (cudaStream_t)stream;
    std::pair<cudaEvent_t, cudaEvent_t> ev{nullptr, nullptr};
    cudaError_t e;
    const bool prof = (flags & FE_PROFILE) != 0;
    if (prof) {
        if (!h->prof_pool.empty()) {
            ev = h->prof_pool.back();
            h->prof_pool.pop_back();
        } else if ((e = cudaEventCreate(&ev.first)) != cudaSuccess || (e = cudaEventCreate(&ev.second)) != cudaSuccess) {
            return cuda_fail(h, e, "cudaEventCreate");
        }
        cudaEventRecord(ev.first, st);
    }
    if ((e = cudaGraphLaunch(h->graphs[graph].second, st)) != cudaSuccess) return cuda_fail(h, e, "cudaGraphLaunch");
    if (prof) {
        cudaEventRecord(ev.second, st);
        h->prof_events.push_back(ev);
    }
    h->last_stream = st;
    h->pending = 1;
    if (flags & FE_ASYNC) return FE_OK;
    return fe_sync(h);
}

int fe_graph_destroy(fe_handle* h, int32_t graph) {
    if (!h || graph < 0 || graph >= (int32_t)h->graphs.size()) return FE_ERR_ARG;
    if (h->pending) fe_sync(h);
    auto& g = h->graphs[graph];
    if (g.second) cudaGraphExecDestroy(g.second);
    if (g.first) cudaGraphDestroy(g.first);
    g = {nullptr, nullptr};
    return FE_OK;
}

int fe_autotune(fe_handle* h, const fe_assemble_params* p, double* nzval, double* f, int32_t n_candidates,
                const int32_t* stage_caps, int32_t reps, fe_tune_result* out) {
    static const int32_t defaults[] = {6144, 8192, 10240, 12288, 16384, 24576};
    if (!h || !p || !out) return FE_ERR_ARG;
    if (h->capturing) return set_error(h, FE_ERR_STATE, "autotune during a capture");
    h->plan_pinned = true;  // the candidates are timed as planned, and the choice stands
    if (!stage_caps || n_candidates < 1) {
        stage_caps = defaults;
        n_candidates = (int32_t)(sizeof(defaults) / sizeof(defaults[0]));
    }
    if (n_candidates > FE_TUNE_MAX) n_candidates = FE_TUNE_MAX;
    if (reps < 1) reps = 3;
    *out = fe_tune_result{};
    if (h->pending) fe_sync(h);
    // forms: the one the call names, else every assignment of the subdomains (cell types) to
    // the fused or the two-phase form (bit s of a mask: subdomain s two-phase)
    const int n_sub = (int)h->hp.subs.size();
    const unsigned all = (1u << n_sub) - 1u;
    std::vector<unsigned> masks;
    if (p->flags & FE_TWO_PHASE) masks = {all};
    else if (p->flags & FE_FUSED) masks = {0u};
    else
        for (unsigned m = 0; m <= all; ++m) masks.push_back(m);
    cudaStream_t st = (cudaStream_t)p->stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fe_assemble_params q = *p;
    q.flags = (q.flags & ~(uint32_t)(FE_PROFILE | FE_TWO_PHASE | FE_FUSED)) | FE_ASYNC;
    double best_ms = 1e300;
    int32_t best_cap = h->stage_cap;
    unsigned best_mask = 0;
    int rc = FE_OK;
    for (int32_t k = 0; k < n_candidates && rc == FE_OK; ++k) {
        out->stage_cap[k] = stage_caps[k];
        out->ms[k] = -1.0;
        PlanOptions opt;
        opt.stage_cap = stage_caps[k];
        Error err;
        Plan pl;
        if (build_plan(h->hp, opt, pl, err) != FE_OK || check_plan(h->hp, pl, err) != FE_OK) continue;
        h->plan = std::move(pl);
        cudaError_t ce = install_plan(h);
        if (ce != cudaSuccess) { rc = cuda_fail(h, ce, "autotune: upload plan"); break; }
        h->stage_cap = opt.stage_cap;
        out->n_tiles[k] = h->plan.n_tiles;
        out->n_cell_visits[k] = h->plan.visits;
        for (const unsigned m : masks) {
            h->force_on = true;
            h->force_mask = m;
            // one warm-up, then reps timed assemblies; a form whose tiles do not fit shared
            // memory is skipped
            if (fe_assemble(h, &q, nzval, f) != FE_OK || fe_sync(h) != FE_OK) {
                h->last = fe_error_info{};
                continue;
            }
            cudaEventRecord(e0, st);
            for (int32_t r = 0; r < reps && rc == FE_OK; ++r) rc = fe_assemble(h, &q, nzval, f);
            cudaEventRecord(e1, st);
            if (rc != FE_OK) break;
            rc = fe_sync(h);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            const double per = ms / reps;
            if (out->ms[k] < 0 || per < out->ms[k]) {
                out->ms[k] = per;
                out->form_mask[k] = m;
            }
            if (per < best_ms) {
                best_ms = per;
                best_cap = stage_caps[k];
                best_mask = m;
            }
        }
        h->force_on = false;
    }
    h->force_on = false;
    out->n_candidates = n_candidates;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != FE_OK) return rc;
    if (best_ms == 1e300) return set_error(h, FE_ERR_UNSUPPORTED, "autotune: no candidate ran");
    // keep the fastest plan and form
    if (best_cap != h->stage_cap) {
        PlanOptions opt;
        opt.stage_cap = best_cap;
        Error err;
        Plan pl;
        if (build_plan(h->hp, opt, pl, err) != FE_OK || check_plan(h->hp, pl, err) != FE_OK)
            return set_error(h, FE_ERR_ARG, "autotune: rebuilding the chosen plan failed");
        h->plan = std::move(pl);
        cudaError_t ce = install_plan(h);
        if (ce != cudaSuccess) return cuda_fail(h, ce, "autotune: upload plan");
        h->stage_cap = best_cap;
    }
    h->tuned_valid = true;
    h->tuned_phys = p->physics;
    h->tuned_prec = p->precision;
    h->tuned_mask = best_mask;
    out->best_stage_cap = best_cap;
    out->best_ms = best_ms;
    out->best_form_mask = best_mask;
    return FE_OK;
}

int fe_kernel_time(fe_handle* h, double* total_ms, int64_t* launches) {
    if (!h || !total_ms || !launches) return FE_ERR_ARG;
    double sum = 0;
    for (auto& ev : h->prof_events) {
        cudaError_t e = cudaEventSynchronize(ev.second);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventSynchronize");
        float ms = 0;
        cudaEventElapsedTime(&ms, ev.first, ev.second);
        sum += ms;
        h->prof_pool.push_back(ev);
    }
    *launches = (int64_t)h->prof_events.size();
    *total_ms = sum;
    h->prof_events.clear();
    return FE_OK;
}

int fe_last_error(const fe_handle* h, fe_error_info* out) {
    if (!out) return FE_ERR_ARG;
    *out = h ? h->last : g_create_error;
    return FE_OK;
}

int fe_get_info(const fe_handle* h, fe_info* out) {
    if (!h || !out) return FE_ERR_ARG;
    out->n_cells = h->hp.n_cells;
    out->ndofs = h->hp.ndofs;
    out->nnz = h->hp.nnz;
    out->n_tiles = h->plan.n_tiles;
    out->n_cell_visits = h->plan.visits;
    out->n_items = h->plan.items;
    out->max_record_bytes = h->plan.max_rec;
    out->max_tile_nodes = h->plan.max_nodes;
    out->max_stage_values = h->plan.max_stage;
    out->max_out_doubles = h->plan.max_out;
    out->stage_cap = h->stage_cap;
    out->flagged_cells = h->flagged;
    out->device_bytes = h->mem.bytes();
    out->create_seconds = h->create_seconds;
    return FE_OK;
}

int fe_get_index_map(const fe_handle* h, int64_t cell, int64_t* positions) {
    if (!h || !positions) return FE_ERR_ARG;
    const HostProblem& hp = h->hp;
    if (cell < 1 || cell > hp.n_cells) return FE_ERR_BOUNDS;
    const int s = hp.cell_sub[cell - 1];
    if (s < 0) return FE_ERR_ARG;
    const HostSub& hs = hp.subs[s];
    const int64_t k = hp.cell_local[cell - 1];
    const int nc = hp.nc, nb = hs.nb, ld = nb * nc;
    for (int j = 0; j < nb; ++j) {
        const int64_t n = hs.ents[k * nb + j];
        const int64_t c0 = hp.colptr[nc * n] - 1;
        const int64_t L = hp.colptr[nc * n + 1] - hp.colptr[nc * n];
        for (int i = 0; i < nb; ++i) {
            const size_t t = ((size_t)k * nb + j) * nb + i;
            const int r = hs.wide_rank ? (hs.rank16[t] == 0xFFFF ? -1 : hs.rank16[t]) : (hs.rank8[t] == 255 ? -1 : hs.rank8[t]);
            for (int b = 0; b < nc; ++b)
                for (int a = 0; a < nc; ++a)
                    positions[(int64_t)(j * nc + b) * ld + (i * nc + a)] = r < 0 ? 0 : c0 + b * L + (int64_t)nc * r + a + 1;
        }
    }
    return FE_OK;
}

// ---------------------------------------------------------------------------------------
// Dirichlet constraints (apply!, apply_zero!)
// ---------------------------------------------------------------------------------------
int fe_dirichlet_create(fe_handle* h, const int64_t* rowval, int64_t n_prescribed, const int64_t* prescribed,
                        fe_dirichlet** out) {
    if (!h || !out || (n_prescribed > 0 && (!prescribed || !rowval)) || n_prescribed < 0) return FE_ERR_ARG;
    *out = nullptr;
    const HostProblem& hp = h->hp;
    const int64_t n = hp.ndofs;
    const int64_t* cp = hp.colptr.data();
    // the prescribed dofs of a closed ConstraintHandler: ascending, unique, in range
    for (int64_t i = 0; i < n_prescribed; ++i) {
        if (prescribed[i] < 1 || prescribed[i] > n) return set_error(h, FE_ERR_BOUNDS, "prescribed dof out of range");
        if (i && prescribed[i] <= prescribed[i - 1]) return set_error(h, FE_ERR_ARG, "prescribed dofs must be ascending and unique");
    }
    std::vector<char> isc((size_t)n, 0);
    for (int64_t i = 0; i < n_prescribed; ++i) isc[prescribed[i] - 1] = 1;
    // diagonal positions (binary search: rowval ascending within a column), row bounds
    std::vector<int64_t> diag((size_t)n, -1);
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t c = 0; c < n; ++c) {
        int64_t lo = cp[c] - 1, hi = cp[c + 1] - 1;
        for (int64_t j = lo; j < hi; ++j)
            if (rowval[j] < 1 || rowval[j] > n || (j > lo && rowval[j] <= rowval[j - 1])) bad = 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi) / 2;
            if (rowval[mid] < c + 1) lo = mid + 1;
            else hi = mid;
        }
        if (lo < cp[c + 1] - 1 && rowval[lo] == c + 1) diag[c] = lo;
    }
    if (bad) return set_error(h, FE_ERR_BOUNDS, "rowval out of range or not ascending within a column");
    std::vector<int64_t> pd0((size_t)n_prescribed), pdiag((size_t)n_prescribed);
    for (int64_t i = 0; i < n_prescribed; ++i) {
        const int64_t d = prescribed[i] - 1;
        pd0[i] = d;
        pdiag[i] = diag[d];
        if (diag[d] < 0) {
            char buf[200];
            std::snprintf(buf, sizeof buf, "You are trying to assemble values in to K[%lld, %lld], but K[%lld, %lld] is missing in the sparsity pattern.",
                          (long long)(d + 1), (long long)(d + 1), (long long)(d + 1), (long long)(d + 1));
            return set_error(h, FE_ERR_PATTERN_MISSING, buf, 0, 0, d + 1, d + 1);
        }
    }
    // entries to zero: every entry of a prescribed column, and the prescribed rows elsewhere
    std::vector<int64_t> zero;
    {
        std::vector<int64_t> cnt((size_t)n + 1, 0);
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < n; ++c) {
            int64_t k = 0;
            for (int64_t j = cp[c] - 1; j < cp[c + 1] - 1; ++j) k += isc[c] || isc[rowval[j] - 1];
            cnt[c + 1] = k;
        }
        for (int64_t c = 0; c < n; ++c) cnt[c + 1] += cnt[c];
        zero.resize((size_t)cnt[n]);
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < n; ++c) {
            int64_t k = cnt[c];
            for (int64_t j = cp[c] - 1; j < cp[c + 1] - 1; ++j)
                if (isc[c] || isc[rowval[j] - 1]) zero[k++] = j;
        }
    }
    // f -= K g: per row, its entries in the prescribed columns, in prescribed order
    std::vector<int64_t> rcount((size_t)n + 1, 0);
    for (int64_t i = 0; i < n_prescribed; ++i)
        for (int64_t j = cp[pd0[i]] - 1; j < cp[pd0[i] + 1] - 1; ++j) ++rcount[rowval[j]];
    std::vector<int64_t> rows, rptr(1, 0);
    std::vector<int64_t> slot((size_t)n, -1);
    for (int64_t r = 0; r < n; ++r)
        if (rcount[r + 1]) {
            slot[r] = (int64_t)rows.size();
            rows.push_back(r);
            rptr.push_back(rptr.back() + rcount[r + 1]);
        }
    std::vector<int64_t> epos((size_t)rptr.back());
    std::vector<int32_t> epi((size_t)rptr.back());
    {
        std::vector<int64_t> fill(rptr.begin(), rptr.end() - 1);
        for (int64_t i = 0; i < n_prescribed; ++i)
            for (int64_t j = cp[pd0[i]] - 1; j < cp[pd0[i] + 1] - 1; ++j) {
                const int64_t k = fill[slot[rowval[j] - 1]]++;
                epos[k] = j;
                epi[k] = (int32_t)i;
            }
    }
    fe_dirichlet* ch = new (std::nothrow) fe_dirichlet();
    if (!ch) return FE_ERR_OOM;
    ch->h = h;
    ch->n = n;
    ch->np = n_prescribed;
    ch->n_rows = (int64_t)rows.size();
    ch->n_zero = (int64_t)zero.size();
    cudaError_t e = cudaSetDevice(h->device);
    if (e == cudaSuccess) e = ch->upload(&ch->pd0, pd0.data(), pd0.size());
    if (e == cudaSuccess) e = ch->upload(&ch->diag, diag.data(), diag.size());
    if (e == cudaSuccess) e = ch->upload(&ch->pdiag, pdiag.data(), pdiag.size());
    if (e == cudaSuccess) e = ch->upload(&ch->zero, zero.data(), zero.size());
    if (e == cudaSuccess) e = ch->upload(&ch->rptr, rptr.data(), rptr.size());
    if (e == cudaSuccess) e = ch->upload(&ch->rows, rows.data(), rows.size());
    if (e == cudaSuccess) e = ch->upload(&ch->epos, epos.data(), epos.size());
    if (e == cudaSuccess) e = ch->upload(&ch->epi, epi.data(), epi.size());
    if (e == cudaSuccess) e = ch->upload<double>(&ch->g, nullptr, (size_t)n_prescribed);
    if (e == cudaSuccess) e = ch->upload<double>(&ch->part, nullptr, DIAG_BLOCKS);
    if (e == cudaSuccess) e = ch->upload<double>(&ch->m, nullptr, 1);
    if (e != cudaSuccess) {
        delete ch;
        return cuda_fail(h, e, "dirichlet upload");
    }
    *out = ch;
    return FE_OK;
}

int fe_apply(fe_dirichlet* ch, double* nzval, double* f, const double* inhomogeneities, int32_t applyzero, void* stream) {
    if (!ch || !nzval) return FE_ERR_ARG;
    fe_handle* h = ch->h;
    if (!is_device_ptr(nzval) || (f && !is_device_ptr(f))) return set_error(h, FE_ERR_ARG, "nzval and f must be device memory");
    if (ch->np == 0) return FE_OK;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    const bool inhom = f && !applyzero && inhomogeneities;
    if (inhom && (e = cudaMemcpyAsync(ch->g, inhomogeneities, ch->np * 8, cudaMemcpyDefault, st)) != cudaSuccess)
        return cuda_fail(h, e, "copy inhomogeneities");
    device_attributes(h);
    const unsigned grid = (unsigned)std::max(1, h->n_sm * 4);
    meandiag_partial<<<DIAG_BLOCKS, 256, 0, st>>>(nzval, ch->diag, ch->n, ch->part);
    meandiag_final<<<1, 256, 0, st>>>(ch->part, DIAG_BLOCKS, ch->n, ch->m);
    if (inhom && ch->n_rows) apply_rows<<<grid, 256, 0, st>>>(f, nzval, ch->rptr, ch->rows, ch->epos, ch->epi, ch->g, ch->n_rows);
    if (ch->n_zero) apply_zero_entries<<<grid, 256, 0, st>>>(nzval, ch->zero, ch->n_zero);
    apply_diag<<<grid, 256, 0, st>>>(nzval, f, ch->pdiag, ch->pd0, ch->g, ch->m, ch->np, applyzero || !inhomogeneities ? 1 : 0);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(h, e, "apply kernels");
    return FE_OK;
}

void fe_dirichlet_destroy(fe_dirichlet* ch) { delete ch; }

int fe_element_operator_create(fe_handle* h, const fe_element_layout* layout, int32_t precision, fe_element_operator** out) {
    if (!h || !layout || !out) return FE_ERR_ARG;
    *out = nullptr;
    if (precision != FE_PREC_MIXED && precision != FE_PREC_FP64) return set_error(h, FE_ERR_ARG, "unknown precision");
    const HostProblem& hp = h->hp;
    if (hp.ndofs >= INT32_MAX || hp.n_cells >= INT32_MAX) return set_error(h, FE_ERR_UNSUPPORTED, "more than 2^31 - 1 dofs or cells");
    fe_element_operator* op = new (std::nothrow) fe_element_operator();
    if (!op) return FE_ERR_OOM;
    op->h = h;
    op->fp64 = precision == FE_PREC_FP64;
    for (int k = 0; k < 3; ++k) op->ks[k] = layout->ke_stride[k];
    op->rows = op->ks[0] != 1;
    op->ndofs = hp.ndofs;
    int64_t total = 0;
    op->subs.resize(hp.subs.size());
    for (size_t s = 0; s < hp.subs.size(); ++s) {
        fe_element_operator::Sub& os = op->subs[s];
        os.n = hp.subs[s].nb * hp.subs[s].nc;
        os.n_cells = hp.subs[s].n_cells;
        os.off = total;
        if (os.n_cells && !matvec_supported(os.n)) {
            delete op;
            return set_error(h, FE_ERR_UNSUPPORTED, "no element product compiled for this number of dofs per cell");
        }
        total += (int64_t)os.n * os.n_cells;
    }
    if (total >= INT32_MAX) {
        delete op;
        return set_error(h, FE_ERR_UNSUPPORTED, "more than 2^31 - 1 (cell, dof) pairs");
    }
    // dof -> scratch positions, in ascending cell order (a counting sort over the cells)
    std::vector<int64_t> ptr((size_t)hp.ndofs + 1, 0);
    for (int64_t c = 0; c < hp.n_cells; ++c) {
        const int s = hp.cell_sub[c];
        if (s < 0) continue;
        const int64_t* cd = hp.cell_dofs.data() + hp.cell_dofs_off[c] - 1;
        for (int I = 0; I < op->subs[s].n; ++I) ++ptr[cd[I]];
    }
    for (int64_t d = 0; d < hp.ndofs; ++d) ptr[d + 1] += ptr[d];
    std::vector<int32_t> inc((size_t)ptr[hp.ndofs]);
    {
        std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
        for (int64_t c = 0; c < hp.n_cells; ++c) {
            const int s = hp.cell_sub[c];
            if (s < 0) continue;
            const fe_element_operator::Sub& os = op->subs[s];
            const int64_t k = hp.cell_local[c];
            const int64_t* cd = hp.cell_dofs.data() + hp.cell_dofs_off[c] - 1;
            for (int I = 0; I < os.n; ++I)
                inc[fill[cd[I] - 1]++] = (int32_t)(os.off + (op->rows ? k * os.n + I : I * os.n_cells + k));
        }
    }
    cudaError_t e = cudaSetDevice(h->device);
    for (size_t s = 0; s < hp.subs.size() && e == cudaSuccess; ++s) {
        fe_element_operator::Sub& os = op->subs[s];
        const HostSub& hs = hp.subs[s];
        std::vector<int32_t> dofs((size_t)os.n * os.n_cells);
        for (int64_t k = 0; k < os.n_cells; ++k) {
            const int64_t* cd = hp.cell_dofs.data() + hp.cell_dofs_off[hs.cellid[k]] - 1;
            for (int I = 0; I < os.n; ++I)
                dofs[op->rows ? (size_t)k * os.n + I : (size_t)I * os.n_cells + k] = (int32_t)(cd[I] - 1);
        }
        e = op->upload(&os.cells, hs.cellid.data(), (size_t)os.n_cells);
        if (e == cudaSuccess) e = op->upload(&os.dofs, dofs.data(), dofs.size());
    }
    if (e == cudaSuccess) e = op->upload(&op->ptr, ptr.data(), ptr.size());
    if (e == cudaSuccess) e = op->upload(&op->inc, inc.data(), inc.size());
    if (e == cudaSuccess) {
        if (op->fp64)
            e = op->upload<double>((double**)&op->ye, nullptr, (size_t)total);
        else
            e = op->upload<float>((float**)&op->ye, nullptr, (size_t)total);
    }
    if (e != cudaSuccess) {
        delete op;
        return cuda_fail(h, e, "element operator upload");
    }
    *out = op;
    return FE_OK;
}

int fe_element_matvec(fe_element_operator* op, const void* ke, const double* u, double* y, uint32_t flags, void* stream) {
    if (!op || !ke || !u || !y) return FE_ERR_ARG;
    fe_handle* h = op->h;
    if (!is_device_ptr(ke) || !is_device_ptr(u) || !is_device_ptr(y)) return set_error(h, FE_ERR_ARG, "ke, u and y must be device memory");
    cudaStream_t st = (cudaStream_t)stream;
    device_attributes(h);
    cudaError_t e = cudaSuccess;
    for (const fe_element_operator::Sub& os : op->subs) {
        if (!os.n_cells) continue;
        // threads per cell: products_split(n) (128-thread blocks of 128 / split cells), or a warp
        // (256-thread blocks, 8 cells each)
        const int64_t per_block = op->rows ? 8 : 128 / (op->fp64 ? products_split<double>(os.n) : products_split<float>(os.n));
        const int64_t blocks = (os.n_cells + per_block - 1) / per_block;
        const int64_t cap = (int64_t)h->n_sm * (op->rows ? 8 : 16);
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, cap));
        if (op->fp64)
            e = launch_products<double>(os.n, op->rows, grid, st, (const double*)ke, op->ks, os.cells, os.dofs, os.n_cells, u,
                                        (double*)op->ye + os.off);
        else
            e = launch_products<float>(os.n, op->rows, grid, st, (const float*)ke, op->ks, os.cells, os.dofs, os.n_cells, u,
                                       (float*)op->ye + os.off);
        if (e != cudaSuccess) return cuda_fail(h, e, "element products");
    }
    if (op->ndofs) {
        const int64_t blocks = (op->ndofs + 255) / 256;
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)h->n_sm * 8));
        const int fz = (flags & FE_FILLZERO) ? 1 : 0;
        if (op->fp64)
            dof_gather<double><<<grid, 256, 0, st>>>((const double*)op->ye, op->ptr, op->inc, op->ndofs, fz, y);
        else
            dof_gather<float><<<grid, 256, 0, st>>>((const float*)op->ye, op->ptr, op->inc, op->ndofs, fz, y);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(h, e, "dof gather");
    }
    return FE_OK;
}

void fe_element_operator_destroy(fe_element_operator* op) { delete op; }

int fe_facet_set_create(fe_handle* h, const fe_facet_desc* d, fe_facet_set** out) {
    if (!h || !d || !out || d->n_facets < 0 || (d->n_facets > 0 && (!d->cells || !d->facets))) return FE_ERR_ARG;
    *out = nullptr;
    const HostProblem& hp = h->hp;
    if (d->n_qp < 1 || d->n_qp > 32 || d->n_ref_facets < 1 || !d->qr_weights || !d->N || !d->dMdxi)
        return set_error(h, FE_ERR_ARG, "facet tables: 1 <= n_qp <= 32 points per facet and all tables required");
    // every facet's cell in one subdomain
    int sub = -1;
    for (int64_t k = 0; k < d->n_facets; ++k) {
        const int64_t c = d->cells[k] - 1;
        if (c < 0 || c >= hp.n_cells || hp.cell_sub[c] < 0) return set_error(h, FE_ERR_BOUNDS, "facet cell out of range or in no subdomain");
        if (d->facets[k] < 1 || d->facets[k] > d->n_ref_facets) return set_error(h, FE_ERR_BOUNDS, "local facet number out of range");
        if (sub < 0) sub = hp.cell_sub[c];
        else if (hp.cell_sub[c] != sub) return set_error(h, FE_ERR_UNSUPPORTED, "the facets' cells must belong to one subdomain");
    }
    if (sub < 0) sub = 0;
    const HostSub& hs = hp.subs[sub];
    fe_facet_set* fs = new (std::nothrow) fe_facet_set();
    if (!fs) return FE_ERR_OOM;
    FacetArgs& A = fs->args;
    A.n = d->n_facets;
    A.nf = d->n_ref_facets;
    A.nqp = d->n_qp;
    A.nb = hs.nb;
    A.ng = hs.ng;
    A.nc = hs.nc;
    A.dim = hp.dim;
    A.x = h->base.xd;
    const int nbf = hs.nb * hs.nc;
    std::vector<double> tang((size_t)A.nf * 6);
    for (int f = 0; f < A.nf; ++f)
        if (!facet_tangent_table(hs.cell_type, f + 1, tang.data() + (size_t)f * 6)) {
            delete fs;
            return set_error(h, FE_ERR_UNSUPPORTED, "no facet normals for this cell type / facet count");
        }
    std::vector<int32_t> nodes((size_t)A.n * A.ng), fnr((size_t)A.n), cid((size_t)A.n);
    std::vector<int64_t> dofs((size_t)A.n * nbf);
    for (int64_t k = 0; k < A.n; ++k) {
        const int64_t c = d->cells[k] - 1;
        const int64_t kk = hp.cell_local[c];
        for (int j = 0; j < A.ng; ++j) nodes[k * A.ng + j] = hs.conn[kk * A.ng + j];
        fnr[k] = d->facets[k] - 1;
        cid[k] = (int32_t)c;
        const int64_t* cd = hp.cell_dofs.data() + hp.cell_dofs_off[c] - 1;
        for (int I = 0; I < nbf; ++I) dofs[k * nbf + I] = cd[I] - 1;
    }
    // per dof, its (facet, entry) positions in facet order
    std::vector<int64_t> cnt((size_t)hp.ndofs + 1, 0);
    for (int64_t t = 0; t < (int64_t)dofs.size(); ++t) ++cnt[dofs[t] + 1];
    std::vector<int64_t> rows, rptr(1, 0), slot((size_t)hp.ndofs, -1);
    for (int64_t r = 0; r < hp.ndofs; ++r)
        if (cnt[r + 1]) {
            slot[r] = (int64_t)rows.size();
            rows.push_back(r);
            rptr.push_back(rptr.back() + cnt[r + 1]);
        }
    std::vector<int64_t> epos((size_t)rptr.back());
    {
        std::vector<int64_t> fill(rptr.begin(), rptr.end() - 1);
        for (int64_t t = 0; t < (int64_t)dofs.size(); ++t) epos[fill[slot[dofs[t]]]++] = t;
    }
    fs->h = h;
    fs->n_rows = (int64_t)rows.size();
    const size_t tq = (size_t)A.nf * A.nqp;
    cudaError_t e = cudaSetDevice(h->device);
    int32_t *dn = nullptr, *df = nullptr, *dc = nullptr;
    double *dw = nullptr, *dN = nullptr, *dM = nullptr, *dt = nullptr, *dcon = nullptr;
    if (e == cudaSuccess) e = fs->upload(&dn, nodes.data(), nodes.size());
    if (e == cudaSuccess) e = fs->upload(&df, fnr.data(), fnr.size());
    if (e == cudaSuccess) e = fs->upload(&dc, cid.data(), cid.size());
    if (e == cudaSuccess) e = fs->upload(&dw, d->qr_weights, tq);
    if (e == cudaSuccess) e = fs->upload(&dN, d->N, tq * A.nb);
    if (e == cudaSuccess) e = fs->upload(&dM, d->dMdxi, tq * A.ng * A.dim);
    if (e == cudaSuccess) e = fs->upload(&dt, tang.data(), tang.size());
    if (e == cudaSuccess) e = fs->upload<double>(&dcon, nullptr, (size_t)A.n * nbf);
    if (e == cudaSuccess) e = fs->upload(&fs->rptr, rptr.data(), rptr.size());
    if (e == cudaSuccess) e = fs->upload(&fs->rows, rows.data(), rows.size());
    if (e == cudaSuccess) e = fs->upload(&fs->epos, epos.data(), epos.size());
    if (e == cudaSuccess) e = fs->upload<DevStatus>(&fs->status, nullptr, 1);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&fs->status_h, sizeof(DevStatus));
    if (e != cudaSuccess) {
        delete fs;
        return cuda_fail(h, e, "facet set upload");
    }
    A.nodes = dn;
    A.fnr = df;
    A.cellid = dc;
    A.w = dw;
    A.N = dN;
    A.dM = dM;
    A.tang = dt;
    A.contrib = dcon;
    A.status = fs->status;
    *out = fs;
    return FE_OK;
}

int fe_assemble_facet_load(fe_facet_set* fs, double pressure, const double* traction, uint32_t flags, double* f, void* stream) {
    if (!fs || !f) return FE_ERR_ARG;
    fe_handle* h = fs->h;
    if (!is_device_ptr(f)) return set_error(h, FE_ERR_ARG, "f must be device memory");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    FacetArgs A = fs->args;
    A.pressure = pressure;
    for (int a = 0; a < 3; ++a) A.t[a] = traction ? traction[a] : 0.0;
    if ((flags & FE_FILLZERO) && (e = cudaMemsetAsync(f, 0, h->hp.ndofs * 8, st)) != cudaSuccess) return cuda_fail(h, e, "fill zero");
    if ((e = cudaMemsetAsync(fs->status, 0xFF, 2 * sizeof(unsigned long long), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(&fs->status->flagged, 0, 2 * sizeof(unsigned int), st)) != cudaSuccess)
        return cuda_fail(h, e, "status reset");
    device_attributes(h);
    if (A.n > 0) {
        const unsigned g1 = (unsigned)std::min<int64_t>((A.n + FACET_WARPS - 1) / FACET_WARPS, (int64_t)h->n_sm * 16);
        facet_contrib<<<g1, 32 * FACET_WARPS, 0, st>>>(A);
        const unsigned g2 = (unsigned)std::max<int64_t>(1, std::min<int64_t>((fs->n_rows + 255) / 256, (int64_t)h->n_sm * 8));
        if (fs->n_rows) facet_gather<<<g2, 256, 0, st>>>(f, A.contrib, fs->rptr, fs->rows, fs->epos, fs->n_rows);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(h, e, "facet kernels");
    if ((e = cudaMemcpyAsync(fs->status_h, fs->status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(h, e, "status read");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(h, e, "cudaStreamSynchronize");
    if (fs->status_h->detj_key != ~0ull) {
        const int64_t cell = (int64_t)(fs->status_h->detj_key >> 32) + 1;
        char buf[120];
        std::snprintf(buf, sizeof buf, "det(J) is not positive on a facet of cell %lld", (long long)cell);
        return set_error(h, FE_ERR_DETJ, buf, cell, 0.0);
    }
    return FE_OK;
}

void fe_facet_set_destroy(fe_facet_set* fs) { delete fs; }

}  // extern "C"

// ---------------------------------------------------------------------------------------
// fe_assemble_noalloc: the same assembly without any device allocation, for callers that
// cannot allocate (see the declaration in include/ferrite_gb300.h). The FP32 copies of u and
// of the per-cell factors live in one file-scope device array; its device address is looked
// up once per device on the first call there.
// ---------------------------------------------------------------------------------------
namespace {

constexpr int64_t NOALLOC_SCRATCH_FLOATS = (int64_t)1 << 22;  // 16 MiB per device
static __device__ __align__(256) float g_noalloc_scratch[NOALLOC_SCRATCH_FLOATS];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
float* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on `device`, which must be the current device (the
// symbol resolves on whichever device is current); looked up once per device.
cudaError_t noalloc_scratch(int device, float** out) {
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    int cur = -1;
    const cudaError_t ce = cudaGetDevice(&cur);
    if (ce != cudaSuccess) return ce;
    if (cur != device) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        float* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[device] = ptr;
    }
    *out = g_noalloc_ptr[device];
    return cudaSuccess;
}

__global__ void noalloc_to_float(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = (float)in[k];
}

}  // namespace

extern "C" int fe_assemble_noalloc(fe_handle* h, const fe_assemble_params* p, double* nzval, double* f) {
    if (!h || !p) return FE_ERR_ARG;
    const HostProblem& hp = h->hp;
    const int nc = hp.nc;
    int phys = 0;
    switch (p->physics) {
        case FE_HEAT:
            if (nc != 1) return set_error(h, FE_ERR_ARG, "FE_HEAT needs a scalar field");
            phys = PHYS_HEAT;
            break;
        case FE_LINEAR_ELASTIC:
            if (nc != hp.dim) return set_error(h, FE_ERR_ARG, "FE_LINEAR_ELASTIC needs a dim-component field");
            phys = PHYS_ELASTIC;
            break;
        case FE_NEO_HOOKE:
            if (nc != 3 || hp.dim != 3) return set_error(h, FE_ERR_ARG, "FE_NEO_HOOKE needs a 3-component field in 3D");
            if (!p->u) return set_error(h, FE_ERR_ARG, "FE_NEO_HOOKE needs u");
            phys = PHYS_NEO;
            break;
        default:
            return set_error(h, FE_ERR_ARG, "unknown physics");
    }
    if (p->precision != FE_PREC_MIXED && p->precision != FE_PREC_FP64) return set_error(h, FE_ERR_ARG, "unknown precision");
    if (p->flags & FE_PROFILE) return set_error(h, FE_ERR_ARG, "fe_assemble_noalloc does not profile (events are resources)");
    const bool fp64 = p->precision == FE_PREC_FP64;
    const bool do_k = !(p->flags & FE_NO_K), do_f = !(p->flags & FE_NO_F);
    // every buffer must already be device memory: host buffers would need staging copies
    if (do_k && !is_device_ptr(nzval)) return set_error(h, FE_ERR_ARG, "fe_assemble_noalloc: nzval must be device memory");
    if (do_f && !is_device_ptr(f)) return set_error(h, FE_ERR_ARG, "fe_assemble_noalloc: f must be device memory");
    if (p->u && !is_device_ptr(p->u)) return set_error(h, FE_ERR_ARG, "fe_assemble_noalloc: u must be device memory");
    if (p->cell_scale && !is_device_ptr(p->cell_scale))
        return set_error(h, FE_ERR_ARG, "fe_assemble_noalloc: cell_scale must be device memory");
    const int64_t need = (phys == PHYS_NEO ? hp.ndofs : 0) + (p->cell_scale ? hp.n_cells : 0);
    if (!fp64 && need > NOALLOC_SCRATCH_FLOATS) {
        char buf[200];
        std::snprintf(buf, sizeof buf,
                      "fe_assemble_noalloc: needs %lld scratch floats (u and cell factors in FP32), the static maximum is %lld",
                      (long long)need, (long long)NOALLOC_SCRATCH_FLOATS);
        return set_error(h, FE_ERR_ARG, buf);
    }
    if (h->capturing) return set_error(h, FE_ERR_STATE, "fe_assemble_noalloc: fe_graph_capture is open on this handle");
    cudaStream_t st = (cudaStream_t)p->stream;
    if (!(p->flags & FE_ASYNC)) {
        // a synchronous call ends by waiting for its stream, which a capturing stream refuses
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
            return set_error(h, FE_ERR_STATE, "fe_assemble_noalloc: the stream is capturing; a synchronous call would wait on it");
    }
    if (h->pending) {
        // an earlier FE_ASYNC assembly's error is reported here, before this call replaces it
        const int rc = fe_sync(h);
        if (rc != FE_OK) return rc;
    }
    const KernelEntry* ke = find_kernel(hp, phys, fp64);
    if (!ke) return set_error(h, FE_ERR_UNSUPPORTED, "no kernel compiled for this element / quadrature / physics combination");
    cudaError_t e;
    // the scratch address and every launch below belong to the handle's device
    if ((e = cudaSetDevice(h->device)) != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    float* scratch = nullptr;
    if ((e = noalloc_scratch(h->device, &scratch)) != cudaSuccess) return cuda_fail(h, e, "cudaGetSymbolAddress");
    KernelArgs A = h->base;
    A.nzval = do_k ? nzval : nullptr;
    A.f = do_f ? f : nullptr;
    A.do_k = do_k;
    A.do_f = do_f;
    A.fillzero = (p->flags & FE_FILLZERO) != 0;
    A.compensated = (p->flags & FE_FP32_SUM) == 0;  // compensated unless plain FP32 sums are asked for
    Physics& ph = A.phys;
    ph = Physics{};
    ph.kind = p->physics;
    ph.p0 = p->p0;
    ph.p1 = p->p1;
    for (int x = 0; x < 3; ++x) ph.body[x] = p->body[x];
    if (p->physics == FE_LINEAR_ELASTIC) {
        const double E = p->p0, nu = p->p1;
        ph.lam = E * nu / ((1 + nu) * (1 - 2 * nu));
        ph.mu = E / (2 * (1 + nu));
    }
    ph.cond_threshold = p->cond_threshold > 0 ? (float)p->cond_threshold : 64.0f;
    ph.p0_f = (float)ph.p0;
    ph.p1_f = (float)ph.p1;
    ph.lam_f = (float)ph.lam;
    ph.mu_f = (float)ph.mu;
    for (int x = 0; x < 3; ++x) ph.body_f[x] = (float)ph.body[x];
    // FP32 inputs in the static scratch: u first, then the per-cell factors. Both are fully
    // overwritten here, so nothing needs clearing between calls.
    int64_t off = 0;
    if (phys == PHYS_NEO) {
        ph.u_d = p->u;
        if (!fp64) {
            noalloc_to_float<<<(unsigned)std::min<int64_t>((hp.ndofs + 255) / 256, 4096), 256, 0, st>>>(p->u, scratch, hp.ndofs);
            ph.u_f = scratch;
            off += hp.ndofs;
        }
    }
    if (p->cell_scale) {
        ph.scale_d = p->cell_scale;
        if (!fp64) {
            noalloc_to_float<<<(unsigned)std::min<int64_t>((hp.n_cells + 255) / 256, 4096), 256, 0, st>>>(p->cell_scale, scratch + off,
                                                                                                        hp.n_cells);
            ph.scale_f = scratch + off;
        } else {
            ph.scale_f = (const float*)ph.scale_d;  // non-null marker; the FP64 kernel reads scale_d
        }
    }
    {
        const int rc = launch_assembly(h, ke, A, fp64, st, nullptr);
        if (rc != FE_OK) return rc;
    }
    if ((e = cudaMemcpyAsync(h->status_h, h->status_d, sizeof(DevStatus), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(h, e, "status read");
    h->last_stream = st;
    h->pending = 1;
    if (p->flags & FE_ASYNC) return FE_OK;
    return fe_sync(h);
}
