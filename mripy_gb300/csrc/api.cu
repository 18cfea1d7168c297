// C ABI of the gbnufft library: plans, bin sort, transform pipelines, CUDA graphs and
// the host-buffer entry points that mirror mripy's NUFFT functions.
//
// Pipelines (all on the caller's stream, no host synchronisation after set_points):
//   type-2   pad_deapod -> FFT -> interp                       (nufft_func.py:741-777)
//   type-1   spread -> FFT -> crop_deapod                       (nufft_func.py:702-738)
//   type-21  pad_deapod -> FFT -> interp(*dcf) -> spread -> FFT -> crop_deapod
//                                                               (nufft_func.py:1261-1330)
// The reference fuses interp and spread per sample (build_grid_3d21); with
// output-stationary spreading a tile needs the interpolated values of every sample
// whose stencil reaches it, so the two run as separate kernels with the sample values
// (n_coil complex per sample) kept in a plan-owned buffer between them.
#include <cub/cub.cuh>
#include <cudaTypedefs.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"
#include "tma.cuh"

using namespace gbn;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

}  // namespace

// lets other translation units report through gbn_last_error
int gbn::record_error(int code, const char *msg) { return fail(code, msg); }

namespace {

#define GBN_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail(e_ == cudaErrorMemoryAllocation ? GBN_ERR_ALLOC : GBN_ERR_CUDA,          \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                     \
    } while (0)

#define GBN_FFT(call)                                                                           \
    do {                                                                                        \
        cufftResult r_ = (call);                                                                \
        if (r_ != CUFFT_SUCCESS) return fail(GBN_ERR_CUFFT, std::string(#call) + " failed, cufftResult " + std::to_string((int)r_)); \
    } while (0)

#define GBN_TRY(call)                  \
    do {                               \
        int s_ = (call);               \
        if (s_ != GBN_OK) return s_;   \
    } while (0)

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    template <typename T>
    T *as() const { return (T *)p; }
};

}  // namespace

struct gbn_plan {
    gbn_plan_desc desc{};
    int dim = 2;
    int m[3] = {1, 1, 1};
    int ns = 0;
    int nf[3] = {1, 1, 1};
    double tau = 0;
    Geom gs{}, gi{};
    int coil_group = 1, threads = 256, interp_threads = 256, max_sub = 256, interp_coil_group = 0;
    int interp_staging = 0;  // 0: tensor copies where the grid allows, 1: thread loads
    int interp_variant = 0;  // 3-D, 8 coils: 0 library choice, 1 interp bins, 2 tensor cores
    int spread_variant = 0;  // 3-D, 8 coils: 0 library choice, 1 warp rows, 2 cubes, 3 tensor cores
    bool spread_items_interleaved = false;  // split tiles' work items interleave (cube kernel)
    int dense_min = kDenseDefault;  // 3-D spread tiles with this many samples use compensated sums (0: never)
    int64_t n_dense_sub = 0;
    int64_t n_split = 0;  // spread tiles covered by more than one subproblem (listed in split_tiles)
    int64_t G = 1, n_inst = 1;
    size_t device_bytes = 0;
    int smem_optin = 0;

    // fixed buffers
    float2 *grid = nullptr;
    float *tab[3] = {nullptr, nullptr, nullptr};
    uint32_t *kstatus = nullptr;  // device status word: bits set by kernels whose bounded waits gave up
    cufftHandle fft = 0;
    bool fft_ok = false;
    // The pruned transform of the composite calls (fft_variant): transforms of the trailing
    // axes over the grid planes inside the image band along x (a plan per run length), and a
    // strided pass along x per instance.  The plans share one work area.
    int fft_variant = 0;  // 0 library choice, 1 the full transform, 2 pruned where it applies
    bool fft_band = false;
    cufftHandle fft_planes[3] = {0, 0, 0};
    int fft_planes_batch[3] = {0, 0, 0};
    int fft_n_planes = 0;
    cufftHandle fft_x = 0;
    bool fft_x_ok = false;
    void *fft_work = nullptr;

    // tensor map of the last grid the TMA interp read (re-encoded when the grid changes)
    CUtensorMap tmap{};
    const void *tmap_grid = nullptr;
    int tmap_cg = 0, tmap_bx = 0, tmap_by = 0;

    // point-dependent buffers (grow-only)
    bool points_set = false;
    int64_t M = 0;
    std::vector<int64_t> traj_off;
    DevBuf traj_off_d, grp_scale, pts, home_key, home_keys_sorted, touch_count, touch_off, home_count,
        iota, home_idx, home_pts, dup_keys, dup_vals, dup_keys_sorted, dup_idx, dup_pts, spread_count,
        spread_tile_off, home_tile_off, nsub, sub_off, nsub_i, sub_off_i, spread_subs, interp_subs, cub_tmp, scratch,
        stage_in, stage_out, stage_w, split_tiles, dense_subs;
    int64_t n_dup = 0, n_spread_sub = 0, n_interp_sub = 0;
    int spread_kernels = 0;   // kernels the last spread launched (split-tile zeroing included)
    uint64_t points_gen = 0;  // bumped by every gbn_set_points: captured graphs hold its buffers

    // solvers: workspace (state, partial sums, residual norms, vectors) and the captured
    // iteration graph of the last solve of each kind (CG, IST, FISTA)
    DevBuf solve_ws;
    DevBuf dcf_ws;  // Pipe-Menon weights (complex samples) while gbn_dcf_pipe_menon runs
    struct SolveGraph {
        cudaGraphExec_t exec = nullptr;
        const void *sens = nullptr;
        gbn_layout sl{};
        const float *dcf = nullptr;
        const void *ws = nullptr;
        uint64_t gen = 0;
        int cap = 0, level = -1;
        float step = 0.f, th = 0.f;
    } solve_graph[3];
};

struct gbn_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// spread-list entries (sample x tile) up to which set_points sizes the list's keys and values
// by a bound and synchronises once (256 MB of keys and values)
constexpr uint64_t kOneSyncEntries = (uint64_t)1 << 25;

int ensure(gbn_plan *p, DevBuf &b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return GBN_OK;
    if (b.p) {
        cudaFree(b.p);
        p->device_bytes -= b.cap;
        b.p = nullptr;
        b.cap = 0;
    }
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        cudaGetLastError();
        return fail(GBN_ERR_ALLOC, "cudaMalloc(" + std::to_string(bytes) + ") failed: " + cudaGetErrorString(e));
    }
    b.cap = bytes;
    p->device_bytes += bytes;
    return GBN_OK;
}

void release(DevBuf &b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
}

int compute_params(int dim, int ms, int mt, int mu, double eps, int max_nspread, int *nspread, int64_t nf[3],
                   double *tau) {
    if (dim < 1 || dim > 3) return fail(GBN_ERR_ARG, "dim must be 1, 2 or 3");
    if (!(eps > 1e-33 && eps < 1e-1)) return fail(GBN_ERR_ARG, "eps must satisfy 1e-33 < eps < 1e-1");
    const int sizes[3] = {ms, dim > 1 ? mt : 1, dim > 2 ? mu : 1};
    for (int d = 0; d < dim; ++d)
        if (sizes[d] < 1) return fail(GBN_ERR_ARG, "image sizes must be >= 1");
    // _compute_{1,2,3}d_grid_params, fft/nufft_func.py:198-249
    const double pi = 3.14159265358979323846;
    const int rat = eps > 1e-11 ? 2 : 3;
    int ns = (int)(-std::log(eps) / (pi * (rat - 1) / (rat - 0.5)) + 0.5);
    if (max_nspread > 0) {
        ns = std::min(ns, max_nspread);
        ns = std::max(ns, 3);
    }
    if (ns < 1) ns = 1;
    if (2 * ns > kMaxW) return fail(GBN_ERR_CAPACITY, "nspread above 20 is not supported");
    for (int d = 0; d < 3; ++d) nf[d] = d < dim ? std::max<int64_t>((int64_t)rat * sizes[d], 2 * ns) : 1;
    const double lambda = ns / (rat * (rat - 0.5));
    *tau = pi * lambda / ((double)ms * ms);
    *nspread = ns;
    return GBN_OK;
}

void make_geom(const gbn_plan *p, const int tile[3], Geom &g) {
    g.dim = p->dim;
    g.ns = p->ns;
    g.W = 2 * p->ns;
    g.ntiles = 1;
    for (int d = 0; d < 3; ++d) {
        g.nf[d] = p->nf[d];
        g.tile[d] = d < p->dim ? std::max(1, std::min(tile[d], p->nf[d])) : 1;
        g.ntile[d] = (g.nf[d] + g.tile[d] - 1) / g.tile[d];
        g.ntiles *= g.ntile[d];
        const double h = 2.0 * 3.14159265358979323846 / p->nf[d];
        g.beta2[d] = d < p->dim ? (float)(h * h / (4.0 * p->tau) * 1.4426950408889634) : 0.f;
    }
    g.G = p->G;
    g.n_coil = (int)p->desc.n_coil;
    g.n_traj = (int)p->desc.n_traj;
}

int pow2_floor(int v) {
    int r = 1;
    while (r * 2 <= v) r *= 2;
    return r;
}

int check_plan(const gbn_plan *p, bool need_points) {
    if (!p) return fail(GBN_ERR_ARG, "null plan");
    if (need_points && !p->points_set) return fail(GBN_ERR_STATE, "gbn_set_points has not been called");
    return GBN_OK;
}

DeapodArgs deapod_args(const gbn_plan *p, bool with_group_scale) {
    DeapodArgs a;
    a.g = p->gs;
    for (int d = 0; d < 3; ++d) {
        a.m[d] = p->m[d];
        a.tab[d] = p->tab[d];
    }
    a.grp_scale = with_group_scale ? p->grp_scale.as<float>() : nullptr;
    return a;
}

int fft_exec(gbn_plan *p, float2 *grid, int direction, cudaStream_t s) {
    NvtxRange range("gbn fft");
    if (!p->fft_ok) return fail(GBN_ERR_STATE, "no FFT plan");
    GBN_FFT(cufftSetStream(p->fft, s));
    GBN_FFT(cufftExecC2C(p->fft, (cufftComplex *)grid, (cufftComplex *)grid,
                         direction < 0 ? CUFFT_FORWARD : CUFFT_INVERSE));
    return GBN_OK;
}

// The FFT of the composite calls.  The pad leaves every grid plane outside the image band
// along x (x in [m - m/2, nf - m/2)) zero, and the crop reads only the band, so:
//   band input (after the pad):   trailing-axes transforms of the band planes, then x;
//   band output (before the crop): x, then trailing-axes transforms of the band planes.
// The other planes' trailing-axes transforms are skipped (zero in and zero out, or never
// read).  Plane g = instance * nf0 + x: instance i's upper band run [nf0 - m/2, nf0) and
// instance i+1's lower run [0, m - m/2) are adjacent, so the band planes form n_inst + 1
// runs of m - m/2, m (n_inst - 1 times) and m/2 planes.  Without a pruned transform
// (fft_variant 1, or where it does not apply) this is the full transform.
int fft_band_exec(gbn_plan *p, float2 *grid, int direction, int band, cudaStream_t s) {
    if (!p->fft_band) return fft_exec(p, grid, direction, s);
    NvtxRange range("gbn fft band");
    const int dirc = direction < 0 ? CUFFT_FORWARD : CUFFT_INVERSE;
    const int64_t nf0 = p->nf[0], P = p->G / nf0;
    const int lo = p->m[0] - p->m[0] / 2, hi = p->m[0] / 2;
    auto planes = [&]() -> int {
        for (int64_t k = 0; k <= p->n_inst; ++k) {
            const int64_t start = k == 0 ? 0 : k * nf0 - hi;
            const int len = k == 0 ? lo : (k == p->n_inst ? hi : lo + hi);
            if (len == 0) continue;
            int j = 0;
            while (j < p->fft_n_planes && p->fft_planes_batch[j] != len) ++j;
            if (j == p->fft_n_planes) return fail(GBN_ERR_INTERNAL, "no FFT plan for a band run");
            cufftComplex *ptr = (cufftComplex *)(grid + start * P);
            GBN_FFT(cufftSetStream(p->fft_planes[j], s));
            GBN_FFT(cufftExecC2C(p->fft_planes[j], ptr, ptr, dirc));
        }
        return GBN_OK;
    };
    auto xpass = [&]() -> int {
        GBN_FFT(cufftSetStream(p->fft_x, s));
        for (int64_t i = 0; i < p->n_inst; ++i) {
            cufftComplex *ptr = (cufftComplex *)(grid + i * p->G);
            GBN_FFT(cufftExecC2C(p->fft_x, ptr, ptr, dirc));
        }
        return GBN_OK;
    };
    if (band == GBN_BAND_INPUT) {
        GBN_TRY(planes());
        return xpass();
    }
    GBN_TRY(xpass());
    return planes();
}

// shared memory a block may take when choosing coils per block: in 3-D two blocks per SM
// (latency hiding) beat more coils per block
size_t smem_budget(const gbn_plan *p) {
    return p->dim == 3 ? std::min<size_t>((size_t)p->smem_optin, 116 * 1024) : (size_t)p->smem_optin;
}

int dir_type1(const gbn_plan *p) { return p->desc.iflag < 0 ? GBN_FFT_FORWARD : GBN_FFT_INVERSE; }
int dir_type2(const gbn_plan *p) { return p->desc.iflag < 0 ? GBN_FFT_INVERSE : GBN_FFT_FORWARD; }

// coils per spread block: the plan's group, capped at the coil count and by shared memory
int spread_cg(const gbn_plan *p) {
    int cg = std::min(p->coil_group, pow2_floor(std::max(1, (int)p->desc.n_coil)));
    while (cg > 1 && spread_smem_bytes(p->gs, cg) > smem_budget(p)) cg /= 2;
    return cg;
}

// the cube or tensor-core kernel runs this plan's spreads; they alone read interleaved work
// items (the tensor-core interp reads them too), so set_points builds them exactly when this
// holds
bool spread_interleaved(const gbn_plan *p) { return spread_reads_interleaved(p->gs, spread_cg(p), p->spread_variant); }

int run_spread(gbn_plan *p, const void *c, gbn_layout L, const float *weight, float2 *grid, cudaStream_t s) {
    NvtxRange range("gbn spread");
    // tiles covered by several work items start from zero; when they are most of the grid
    // (dense trajectories), one memset of the whole grid is cheaper than per-tile blocks
    const bool memset_grid = 2 * p->n_split > (int64_t)p->gs.ntiles * p->gs.n_traj;
    if (memset_grid)
        GBN_CUDA(cudaMemsetAsync(grid, 0, sizeof(float2) * (size_t)p->G * (size_t)p->n_inst, s));
    else
        GBN_CUDA(launch_zero_split(p->gs, p->split_tiles.as<uint32_t>(), p->n_split, grid, s));
    SpreadArgs a;
    a.g = p->gs;
    a.subs = p->spread_subs.as<int4>();
    a.pts = p->dup_pts.as<float4>();
    a.idx = p->dup_idx.as<uint32_t>();
    a.pts_by_sample = p->pts.as<float4>();
    a.c = (const float2 *)c;
    a.c_elem = L.elem_stride;
    a.c_coil = L.coil_stride;
    a.weight = weight;
    a.grid = grid;
    a.any_dense = p->n_dense_sub > 0 ? 1 : 0;
    a.dense_subs = p->dense_subs.as<uint32_t>();
    a.n_dense = p->n_dense_sub;
    a.variant = p->spread_variant;
    a.status = p->kstatus;
    const int cg = spread_cg(p);
    if (spread_smem_bytes(p->gs, cg) > (size_t)p->smem_optin)
        return fail(GBN_ERR_CAPACITY, "spread tile does not fit in shared memory");
    if (p->spread_items_interleaved != spread_interleaved(p))
        return fail(GBN_ERR_INTERNAL, "spread work items do not match the spread kernel");
    GBN_CUDA(launch_spread(a, p->n_spread_sub, cg, p->threads, s));
    p->spread_kernels = (!memset_grid && p->n_split > 0 ? 1 : 0) + spread_kernel_count(a, p->n_spread_sub, cg, p->threads);
    return GBN_OK;
}

// Interp coils per block: the caller's choice, else the group size that pads the coil
// count least (every padded lane still reads the window), counting 2 lanes of fixed cost
// per block: 12 coils -> 3 groups of 4, 8 -> 1 of 8, 5 -> 1 of 8, 3 -> 1 of 4.
int interp_cg(const gbn_plan *p) {
    const int n = std::max(1, (int)p->desc.n_coil);
    int cg = p->interp_coil_group;
    // a caller's group larger than the coil count only pads (e.g. a tuning chosen for 8
    // coils applied to a one-coil plan): cap it at the smallest power of two >= n
    int n_pow2 = 1;
    while (n_pow2 < n) n_pow2 *= 2;
    if (cg > n_pow2) cg = n_pow2;
    if (cg <= 0) {
        int best = 1 << 30;
        for (int cand : {8, 4, 2, 1}) {
            const int cost = ((n + cand - 1) / cand) * (cand + 2);
            if (cost < best) {
                best = cost;
                cg = cand;
            }
        }
    }
    while (cg > 1 && interp_smem_bytes(p->gi, cg, p->interp_threads) > smem_budget(p)) cg /= 2;
    return cg;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against the
// driver library); null when the driver does not provide it
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        else
            cudaGetLastError();
    });
    return fn;
}

// Tensor map of a 2-D plan grid as a 3-D tensor (y innermost, x, instance) of 8-byte
// cells, box BY x BX x cg coils (an item's coils); cached for the last grid pointer and box.  False when the
// grid is not 16-byte aligned, its rows are not a multiple of 16 bytes, or the driver
// lacks the encoder: the caller then uses the thread-staged kernel.
bool grid_tensor_map(gbn_plan *p, const float2 *grid, int cg, const TmaWin &t) {
    if (p->tmap_grid == grid && p->tmap_cg == cg && p->tmap_bx == t.BX && p->tmap_by == t.BY) return true;
    p->tmap_grid = nullptr;
    if ((reinterpret_cast<uintptr_t>(grid) & 15) || (p->nf[1] & 1)) return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)p->nf[1], (cuuint64_t)p->nf[0], (cuuint64_t)p->n_inst};
    const cuuint64_t strides[2] = {(cuuint64_t)p->nf[1] * sizeof(float2),
                                   (cuuint64_t)p->nf[0] * p->nf[1] * sizeof(float2)};
    const cuuint32_t box[3] = {(cuuint32_t)t.BY, (cuuint32_t)t.BX, (cuuint32_t)cg};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(&p->tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<float2 *>(grid), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    p->tmap_grid = grid;
    p->tmap_cg = cg;
    p->tmap_bx = t.BX;
    p->tmap_by = t.BY;
    return true;
}

// 3-D: the grid as a 4-D tensor (z innermost, y, x, instance) of 8-byte cells with the
// plane box BZ x BY x 1 x cg of the plane-streaming interp
bool grid_tensor_map3d(gbn_plan *p, const float2 *grid, int cg, int BY, int BZ) {
    if (p->tmap_grid == grid && p->tmap_cg == cg && p->tmap_bx == BY && p->tmap_by == BZ) return true;
    p->tmap_grid = nullptr;
    if ((reinterpret_cast<uintptr_t>(grid) & 15) || (p->nf[2] & 1)) return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)p->nf[2], (cuuint64_t)p->nf[1], (cuuint64_t)p->nf[0],
                                (cuuint64_t)p->n_inst};
    const cuuint64_t strides[3] = {(cuuint64_t)p->nf[2] * sizeof(float2),
                                   (cuuint64_t)p->nf[1] * p->nf[2] * sizeof(float2),
                                   (cuuint64_t)p->G * sizeof(float2)};
    const cuuint32_t box[4] = {(cuuint32_t)BZ, (cuuint32_t)BY, 1u, (cuuint32_t)cg};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = enc(&p->tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<float2 *>(grid), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    p->tmap_grid = grid;
    p->tmap_cg = cg;
    p->tmap_bx = BY;
    p->tmap_by = BZ;
    return true;
}

// the tensor-core interp runs this plan's interps (on the spread's tiles and work lists)
bool interp_on_tensor_cores(const gbn_plan *p) {
    return p->interp_variant != 1 && interp_mma_applies(p->gs, spread_cg(p));
}

int run_interp(gbn_plan *p, const float2 *grid, void *c, gbn_layout L, const float *weight, cudaStream_t s) {
    NvtxRange range("gbn interp");
    if (interp_on_tensor_cores(p)) {
        MmaInterpArgs m;
        m.g = p->gs;
        m.subs = p->spread_subs.as<int4>();
        m.idx = p->dup_idx.as<uint32_t>();
        m.pts_by_sample = p->pts.as<float4>();
        m.grid = grid;
        m.c = (float2 *)c;
        m.c_elem = L.elem_stride;
        m.c_coil = L.coil_stride;
        m.weight = weight;
        m.M = p->M;
        GBN_CUDA(launch_interp3d_mma(m, p->n_spread_sub, p->kstatus, s));
        return GBN_OK;
    }
    InterpArgs a;
    a.g = p->gi;
    a.subs = p->interp_subs.as<int4>();
    a.pts = p->home_pts.as<float4>();
    a.idx = p->home_idx.as<uint32_t>();
    a.grid = grid;
    a.c = (float2 *)c;
    a.c_elem = L.elem_stride;
    a.c_coil = L.coil_stride;
    a.weight = weight;
    const int cg = interp_cg(p);
    // 2-D: windows staged by tensor copies when the grid admits a tensor map
    TmaWin t{};
    if (p->interp_staging == 0 && tma_window(p->gi, cg, p->n_interp_sub, t) &&
        tma_interp_smem_bytes(t) <= (size_t)p->smem_optin && grid_tensor_map(p, grid, cg * t.passes, t)) {
        GBN_CUDA(launch_interp2d_tma(a, t, p->tmap, cg, p->interp_threads, p->kstatus, s));
        return GBN_OK;
    }
    if (interp_smem_bytes(p->gi, cg, p->interp_threads) > (size_t)p->smem_optin)
        return fail(GBN_ERR_CAPACITY, "interp window does not fit in shared memory");
    // 3-D, 4 or 8 coils per block: planes staged by tensor copies when the grid admits a map
    int BY = 0, BZ = 0;
    if (p->dim == 3 && interp3d_plane_box(p->gi, cg, BY, BZ)) {
        const bool tma = p->interp_staging == 0 && grid_tensor_map3d(p, grid, cg, BY, BZ);
        GBN_CUDA(launch_interp3d_planes(a, p->n_interp_sub, cg, p->interp_threads, tma ? &p->tmap : nullptr,
                                        tma ? p->kstatus : nullptr, s));
        return GBN_OK;
    }
    GBN_CUDA(launch_interp(a, p->n_interp_sub, cg, p->interp_threads, s));
    return GBN_OK;
}

template <typename F>
int cub_call(gbn_plan *p, F f) {
    size_t bytes = 0;
    GBN_CUDA(f(nullptr, bytes));
    GBN_TRY(ensure(p, p->cub_tmp, bytes));
    bytes = p->cub_tmp.cap;
    GBN_CUDA(f(p->cub_tmp.p, bytes));
    return GBN_OK;
}

int key_bits(uint64_t max_key) {
    int b = 1;
    while (b < 32 && (1ull << b) <= max_key) ++b;
    return b;
}

// count -> tile offsets (exclusive), subproblem table
// Work items of one bin geometry, in two phases so that the spread's and the interp's
// totals (and the dense / split counts) come back to the host in one synchronisation.
struct SubsJob {
    const Geom *g;
    uint32_t *count;      // samples per tile
    DevBuf *tile_off;     // their exclusive scan
    DevBuf *nsub;         // work items per tile
    DevBuf *sub_off;      // their exclusive scan
    int every_tile, max_sub;
    uint32_t dense_min;
    uint32_t *n_dense, *n_split;  // device counters (may be null)
    int interleave = 0;           // split tiles' items take every s-th entry
    int64_t T = 0;
};

// scans and per-tile item counts; the last tile's offset and count are copied into last[2]
int subs_count(gbn_plan *p, SubsJob &j, uint32_t last[2], cudaStream_t s) {
    j.T = (int64_t)j.g->ntiles * j.g->n_traj;
    const int64_t T = j.T;
    GBN_TRY(ensure(p, *j.tile_off, sizeof(uint32_t) * T));
    GBN_TRY(ensure(p, *j.nsub, sizeof(uint32_t) * T));
    GBN_TRY(ensure(p, *j.sub_off, sizeof(uint32_t) * (T + 1)));
    uint32_t *toff = j.tile_off->as<uint32_t>(), *ns_ = j.nsub->as<uint32_t>(), *soff = j.sub_off->as<uint32_t>();
    GBN_TRY(cub_call(p, [&](void *tmp, size_t &bytes) {
        return cub::DeviceScan::ExclusiveSum(tmp, bytes, j.count, toff, (int)T, s);
    }));
    GBN_CUDA(launch_count_subs(j.count, T, j.max_sub, j.every_tile, j.dense_min, ns_, j.n_dense, j.n_split, s));
    GBN_TRY(cub_call(p, [&](void *tmp, size_t &bytes) {
        return cub::DeviceScan::ExclusiveSum(tmp, bytes, ns_, soff, (int)T, s);
    }));
    GBN_CUDA(cudaMemcpyAsync(&last[0], soff + (T - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    GBN_CUDA(cudaMemcpyAsync(&last[1], ns_ + (T - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    return GBN_OK;
}

// after the synchronisation: allocate and fill the work items
int subs_build(gbn_plan *p, const SubsJob &j, const uint32_t last[2], DevBuf &subs, uint32_t *split_list,
               uint32_t *split_cursor, uint32_t *dense_list, uint32_t *dense_cursor, int64_t *n_sub_out,
               cudaStream_t s) {
    const int64_t n_sub = (int64_t)last[0] + last[1];
    if (n_sub > 0x7FFFFFFF) return fail(GBN_ERR_CAPACITY, "too many subproblems");
    GBN_TRY(ensure(p, subs, sizeof(int4) * (size_t)std::max<int64_t>(n_sub, 1)));
    GBN_CUDA(launch_build_subs(j.count, j.tile_off->as<uint32_t>(), j.sub_off->as<uint32_t>(), j.T, j.max_sub,
                               j.every_tile, j.dense_min, j.interleave, split_list, split_cursor, dense_list,
                               dense_cursor, subs.as<int4>(), s));
    *n_sub_out = n_sub;
    return GBN_OK;
}

__global__ void k_iota(uint32_t *v, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = (uint32_t)i;
}

int set_points_impl(gbn_plan *p, int dtype, const void *x, const void *y, const void *z, const int64_t *off,
                    cudaStream_t s) {
    NvtxRange range("gbn set_points");
    GBN_TRY(check_plan(p, false));
    const int nt = p->desc.n_traj;
    if (!off) return fail(GBN_ERR_ARG, "traj_offsets is null");
    if (dtype != GBN_COORD_F32 && dtype != GBN_COORD_F64) return fail(GBN_ERR_ARG, "bad coordinate dtype");
    if (off[0] != 0) return fail(GBN_ERR_ARG, "traj_offsets[0] must be 0");
    for (int g = 0; g < nt; ++g)
        if (off[g + 1] < off[g]) return fail(GBN_ERR_ARG, "traj_offsets must be non-decreasing");
    const int64_t M = off[nt];
    if (M >= (int64_t)1 << 31) return fail(GBN_ERR_CAPACITY, "more than 2^31-1 samples");
    const void *src[3] = {x, y, z};
    for (int d = 0; d < p->dim; ++d)
        if (M > 0 && !src[d]) return fail(GBN_ERR_ARG, "coordinate pointer is null");
    p->points_set = false;
    p->M = M;
    p->traj_off.assign(off, off + nt + 1);

    const size_t Mb = (size_t)std::max<int64_t>(M, 1);
    const int64_t Ti = (int64_t)p->gi.ntiles * nt, Ts = (int64_t)p->gs.ntiles * nt;
    GBN_TRY(ensure(p, p->traj_off_d, sizeof(int64_t) * (nt + 1)));
    GBN_TRY(ensure(p, p->grp_scale, sizeof(float) * nt));
    GBN_TRY(ensure(p, p->pts, sizeof(float4) * Mb));
    GBN_TRY(ensure(p, p->home_key, sizeof(uint32_t) * Mb));
    GBN_TRY(ensure(p, p->home_keys_sorted, sizeof(uint32_t) * Mb));
    GBN_TRY(ensure(p, p->touch_count, sizeof(uint32_t) * Mb));
    GBN_TRY(ensure(p, p->touch_off, sizeof(uint64_t) * Mb));
    GBN_TRY(ensure(p, p->home_count, sizeof(uint32_t) * (Ti + 1)));  // + status word
    GBN_TRY(ensure(p, p->iota, sizeof(uint32_t) * Mb));
    GBN_TRY(ensure(p, p->home_idx, sizeof(uint32_t) * Mb));
    GBN_TRY(ensure(p, p->home_pts, sizeof(float4) * Mb));
    GBN_TRY(ensure(p, p->spread_count, sizeof(uint32_t) * Ts));
    GBN_TRY(ensure(p, p->scratch, sizeof(float2) * Mb * (size_t)p->desc.n_coil));

    std::vector<float> gscale(nt);
    for (int g = 0; g < nt; ++g) {
        const int64_t Mg = off[g + 1] - off[g];
        gscale[g] = Mg > 0 ? (float)(1.0 / (double)Mg) : 0.f;
    }
    GBN_CUDA(cudaMemcpyAsync(p->traj_off_d.p, off, sizeof(int64_t) * (nt + 1), cudaMemcpyHostToDevice, s));
    GBN_CUDA(cudaMemcpyAsync(p->grp_scale.p, gscale.data(), sizeof(float) * nt, cudaMemcpyHostToDevice, s));
    GBN_CUDA(cudaMemsetAsync(p->home_count.p, 0, sizeof(uint32_t) * (Ti + 1), s));
    GBN_CUDA(cudaMemsetAsync(p->spread_count.p, 0, sizeof(uint32_t) * Ts, s));

    uint32_t *home_count = p->home_count.as<uint32_t>();
    GBN_CUDA(launch_prep(dtype, x, y, z, M, p->traj_off_d.as<int64_t>(), p->gs, p->gi, p->desc.df,
                         p->pts.as<float4>(), p->home_key.as<uint32_t>(), p->touch_count.as<uint32_t>(),
                         home_count, s));
    uint32_t *tc = p->touch_count.as<uint32_t>();
    uint64_t *to = p->touch_off.as<uint64_t>();
    if (M > 0) {
        GBN_TRY(cub_call(p, [&](void *tmp, size_t &bytes) {
            return cub::DeviceScan::ExclusiveSum(tmp, bytes, tc, to, (int)M, s);
        }));
    }
    // The spread list (one entry per sample and tile its stencil reaches) has E = sum of the
    // touch counts entries.  When a bound on E fits kOneSyncEntries, its keys are written
    // before E is known and the work-item counts are queued behind them, so one host
    // synchronisation returns E, the counts and the status together (set_points on a changing
    // trajectory, as in a differentiable reconstruction, then costs one round trip).  Per axis
    // a W-cell stencil reaches at most ceil((W-1)/T) + 1 tiles, one more when a partial last
    // tile sits at the wrap, and never more than the axis has.
    uint64_t bound = (uint64_t)M;
    for (int d = 0; d < p->dim; ++d) {
        const Geom &g = p->gs;
        const uint64_t per = (uint64_t)((g.W - 1 + g.tile[d] - 1) / g.tile[d] + (g.nf[d] % g.tile[d] ? 2 : 1));
        bound *= std::min<uint64_t>(per, (uint64_t)g.ntile[d]);
    }
    const bool one_sync = M > 0 && bound <= kOneSyncEntries;
    uint32_t *scount = p->spread_count.as<uint32_t>();
    // 3-D: spread tiles with at least dense_min samples (the k-space centre of radial
    // trajectories) accumulate with compensated sums; status word 1 counts their work items,
    // word 2 the split tiles (zeroed before each spread), word 3 is the split list's cursor
    const uint32_t dense_min = p->dim == 3 && p->dense_min > 0 ? (uint32_t)p->dense_min : 0u;
    GBN_TRY(ensure(p, p->split_tiles, sizeof(uint32_t) * (size_t)std::max<int64_t>(Ts, 1)));
    // the plane-streaming 3-D interp holds a chunk of kPlaneSamples samples' state; work
    // items of at most that size stream each window once
    const int interp_max_sub = interp3d_planes_smem(p->gi, interp_cg(p), p->interp_threads) > 0
                                   ? std::min(p->max_sub, kPlaneSamples)
                                   : p->max_sub;
    SubsJob js{&p->gs, scount, &p->spread_tile_off, &p->nsub, &p->sub_off, 1, p->max_sub, dense_min,
               p->kstatus + 1, p->kstatus + 2};
    js.interleave = spread_interleaved(p) ? 1 : 0;
    p->spread_items_interleaved = js.interleave != 0;
    SubsJob ji{&p->gi, home_count, &p->home_tile_off, &p->nsub_i, &p->sub_off_i, 0, interp_max_sub, 0u, nullptr,
               nullptr};
    uint32_t sizes[6] = {0, 0, 0, 0, 0, 0};  // spread last offset / count, interp ditto, dense, split
    auto queue_counts = [&]() -> int {
        GBN_CUDA(cudaMemsetAsync(p->kstatus + 1, 0, 4 * sizeof(uint32_t), s));
        GBN_TRY(subs_count(p, js, sizes, s));
        GBN_TRY(subs_count(p, ji, sizes + 2, s));
        GBN_CUDA(cudaMemcpyAsync(sizes + 4, p->kstatus + 1, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        return GBN_OK;
    };
    if (one_sync) {
        GBN_TRY(ensure(p, p->dup_keys, sizeof(uint32_t) * (size_t)bound));
        GBN_TRY(ensure(p, p->dup_vals, sizeof(uint32_t) * (size_t)bound));
        GBN_CUDA(launch_dup_keys(p->pts.as<float4>(), M, p->traj_off_d.as<int64_t>(), nt, p->gs, to,
                                 p->dup_keys.as<uint32_t>(), p->dup_vals.as<uint32_t>(), scount, s));
        GBN_TRY(queue_counts());
    }
    uint64_t last_off = 0;
    uint32_t last_cnt = 0, status = 0;
    if (M > 0) {
        GBN_CUDA(cudaMemcpyAsync(&last_off, to + (M - 1), sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        GBN_CUDA(cudaMemcpyAsync(&last_cnt, tc + (M - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    }
    GBN_CUDA(cudaMemcpyAsync(&status, home_count + Ti, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    GBN_CUDA(cudaStreamSynchronize(s));
    if (status & 1u) return fail(GBN_ERR_ARG, "non-finite trajectory coordinate");
    const uint64_t E = M > 0 ? last_off + last_cnt : 0;
    if (E >= ((uint64_t)1 << 31)) return fail(GBN_ERR_CAPACITY, "spread list above 2^31 entries");
    if (one_sync && E > bound) return fail(GBN_ERR_INTERNAL, "spread list above its bound");
    p->n_dup = (int64_t)E;
    const size_t Eb = (size_t)std::max<uint64_t>(E, 1);
    GBN_TRY(ensure(p, p->dup_keys, sizeof(uint32_t) * Eb));
    GBN_TRY(ensure(p, p->dup_vals, sizeof(uint32_t) * Eb));
    GBN_TRY(ensure(p, p->dup_keys_sorted, sizeof(uint32_t) * Eb));
    GBN_TRY(ensure(p, p->dup_idx, sizeof(uint32_t) * Eb));
    GBN_TRY(ensure(p, p->dup_pts, sizeof(float4) * Eb));
    if (!one_sync)
        GBN_CUDA(launch_dup_keys(p->pts.as<float4>(), M, p->traj_off_d.as<int64_t>(), nt, p->gs, to,
                                 p->dup_keys.as<uint32_t>(), p->dup_vals.as<uint32_t>(), scount, s));
    if (E > 0) {
        uint32_t *kin = p->dup_keys.as<uint32_t>(), *vin = p->dup_vals.as<uint32_t>();
        uint32_t *kout = p->dup_keys_sorted.as<uint32_t>(), *vout = p->dup_idx.as<uint32_t>();
        const int bits = key_bits((uint64_t)Ts);
        GBN_TRY(cub_call(p, [&](void *tmp, size_t &bytes) {
            return cub::DeviceRadixSort::SortPairs(tmp, bytes, kin, kout, vin, vout, (int)E, 0, bits, s);
        }));
        GBN_CUDA(launch_gather_pts(p->pts.as<float4>(), vout, (int64_t)E, p->dup_pts.as<float4>(), s));
    }
    if (M > 0) {
        k_iota<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(p->iota.as<uint32_t>(), M);
        GBN_CUDA(cudaGetLastError());
        uint32_t *kin = p->home_key.as<uint32_t>(), *vin = p->iota.as<uint32_t>();
        uint32_t *kout = p->home_keys_sorted.as<uint32_t>(), *vout = p->home_idx.as<uint32_t>();
        const int bits = key_bits((uint64_t)Ti);
        GBN_TRY(cub_call(p, [&](void *tmp, size_t &bytes) {
            return cub::DeviceRadixSort::SortPairs(tmp, bytes, kin, kout, vin, vout, (int)M, 0, bits, s);
        }));
        GBN_CUDA(launch_gather_pts(p->pts.as<float4>(), vout, M, p->home_pts.as<float4>(), s));
    }
    if (!one_sync) {
        GBN_TRY(queue_counts());
        GBN_CUDA(cudaStreamSynchronize(s));
    }
    GBN_TRY(ensure(p, p->dense_subs, sizeof(uint32_t) * (size_t)std::max<uint32_t>(sizes[4], 1)));
    GBN_TRY(subs_build(p, js, sizes, p->spread_subs, p->split_tiles.as<uint32_t>(), p->kstatus + 3,
                       p->dense_subs.as<uint32_t>(), p->kstatus + 4, &p->n_spread_sub, s));
    GBN_TRY(subs_build(p, ji, sizes + 2, p->interp_subs, nullptr, nullptr, nullptr, nullptr, &p->n_interp_sub, s));
    const uint32_t counts[2] = {sizes[4], sizes[5]};
    p->n_dense_sub = counts[0];
    p->n_split = counts[1];
    p->points_gen += 1;
    p->points_set = true;
    return GBN_OK;
}

// Whether the composite calls run the pruned transform.  Library choice: 3-D grids of at
// least 2^21 cells per instance (a transform pass moves >= 16 MB per instance there, so the
// 2 n_inst + 1 plan executions of a pruned transform cost little next to it), at most 256
// instances.  fft_variant 2 asks for it wherever the band is narrower than the grid (2-D and
// 3-D, at most 4096 instances).
bool fft_band_wanted(const gbn_plan *p) {
    if (p->fft_variant == 1 || p->dim < 2 || p->m[0] >= p->nf[0] || p->G > 0x7FFFFFFF) return false;
    if (p->fft_variant == 2) return p->n_inst <= 4096;
    return p->dim == 3 && p->G >= ((int64_t)1 << 21) && p->n_inst <= 256;
}

// The pruned transform's plans (used by fft_band_exec): one trailing-axes plan per distinct
// band-run length, batched over the run's planes, and the x pass (stride = plane size,
// batched over the plane's cells), all on one work area.
int make_fft_band(gbn_plan *p) {
    const int lo = p->m[0] - p->m[0] / 2, hi = p->m[0] / 2;
    const int runs[3] = {lo, p->n_inst > 1 ? lo + hi : 0, hi};
    int n_tr[2] = {p->nf[1], p->nf[2]};
    const int P = (int)(p->G / p->nf[0]);
    size_t ws_max = 0;
    auto check = [&](cufftResult r, const char *what) {
        return r == CUFFT_SUCCESS ? GBN_OK
                                  : fail(GBN_ERR_CUFFT, std::string(what) + " failed, cufftResult " + std::to_string((int)r));
    };
    for (int len : runs) {
        if (len == 0) continue;
        bool have = false;
        for (int j = 0; j < p->fft_n_planes; ++j) have |= p->fft_planes_batch[j] == len;
        if (have) continue;
        cufftHandle h = 0;
        GBN_TRY(check(cufftCreate(&h), "cufftCreate"));
        p->fft_planes[p->fft_n_planes] = h;
        p->fft_planes_batch[p->fft_n_planes] = len;
        p->fft_n_planes += 1;
        size_t ws = 0;
        GBN_TRY(check(cufftSetAutoAllocation(h, 0), "cufftSetAutoAllocation"));
        GBN_TRY(check(cufftMakePlanMany(h, p->dim - 1, n_tr, nullptr, 1, P, nullptr, 1, P, CUFFT_C2C, len, &ws),
                      "cufftMakePlanMany (band planes)"));
        ws_max = std::max(ws_max, ws);
    }
    GBN_TRY(check(cufftCreate(&p->fft_x), "cufftCreate"));
    p->fft_x_ok = true;
    int nx[1] = {p->nf[0]};
    size_t ws = 0;
    GBN_TRY(check(cufftSetAutoAllocation(p->fft_x, 0), "cufftSetAutoAllocation"));
    GBN_TRY(check(cufftMakePlanMany(p->fft_x, 1, nx, nx, P, 1, nx, P, 1, CUFFT_C2C, P, &ws),
                  "cufftMakePlanMany (x pass)"));
    ws_max = std::max(ws_max, ws);
    if (ws_max > 0) {
        if (cudaMalloc(&p->fft_work, ws_max) != cudaSuccess) {
            cudaGetLastError();
            p->fft_work = nullptr;
            return fail(GBN_ERR_ALLOC, "FFT work area allocation failed");
        }
        for (int j = 0; j < p->fft_n_planes; ++j)
            GBN_TRY(check(cufftSetWorkArea(p->fft_planes[j], p->fft_work), "cufftSetWorkArea"));
        GBN_TRY(check(cufftSetWorkArea(p->fft_x, p->fft_work), "cufftSetWorkArea"));
        p->device_bytes += ws_max;
    }
    p->fft_band = true;
    return GBN_OK;
}

// releases the pruned transform's plans and work area (the full transform stays)
void drop_fft_band(gbn_plan *p) {
    for (int i = 0; i < p->fft_n_planes; ++i) cufftDestroy(p->fft_planes[i]);
    p->fft_n_planes = 0;
    if (p->fft_x_ok) cufftDestroy(p->fft_x);
    p->fft_x_ok = false;
    if (p->fft_work) cudaFree(p->fft_work);
    p->fft_work = nullptr;
    p->fft_band = false;
}

int plan_create_impl(const gbn_plan_desc *desc, gbn_plan **out) {
    if (!desc || !out) return fail(GBN_ERR_ARG, "null argument");
    *out = nullptr;
    if (desc->n_coil < 1 || desc->n_traj < 1) return fail(GBN_ERR_ARG, "n_coil and n_traj must be >= 1");
    if (!std::isfinite(desc->df)) return fail(GBN_ERR_ARG, "df must be finite");
    gbn_plan *p = new (std::nothrow) gbn_plan();
    if (!p) return fail(GBN_ERR_ALLOC, "host allocation failed");
    p->desc = *desc;
    p->dim = desc->dim;
    int64_t nf64[3];
    int st = compute_params(desc->dim, desc->ms, desc->mt, desc->mu, desc->eps, desc->max_nspread, &p->ns, nf64,
                            &p->tau);
    if (st != GBN_OK) {
        delete p;
        return st;
    }
    p->m[0] = desc->ms;
    p->m[1] = desc->dim > 1 ? desc->mt : 1;
    p->m[2] = desc->dim > 2 ? desc->mu : 1;
    p->G = 1;
    for (int d = 0; d < 3; ++d) {
        p->nf[d] = (int)nf64[d];
        p->G *= nf64[d];
    }
    if (!cells_fit(p->dim, p->nf)) {
        delete p;
        return fail(GBN_ERR_CAPACITY, "oversampled grid too large for the packed cell index");
    }
    p->n_inst = (int64_t)desc->n_coil * desc->n_traj;

    // defaults (the autotuner overrides through desc)
    int dspread[3], dinterp[3];
    if (p->dim == 1) {
        dspread[0] = 1024; dinterp[0] = 1024;
    } else if (p->dim == 2) {
        // measured on GB300 for the 8-coil 512^2 radial workload: 16x32 output tiles keep
        // four spread blocks resident per SM; 16x16 interp bins keep the staged window small
        dspread[0] = 16; dspread[1] = 32;
        dinterp[0] = 16; dinterp[1] = 16;
    } else {
        // warp lanes run along z: 32-cell z rows for the spread tile, 8^3 interp bins
        dspread[0] = 8; dspread[1] = 8; dspread[2] = 32;
        dinterp[0] = 8; dinterp[1] = 8; dinterp[2] = 8;
    }
    int ts[3] = {1, 1, 1}, ti[3] = {1, 1, 1};
    for (int d = 0; d < p->dim; ++d) {
        ts[d] = desc->spread_tile[d] > 0 ? desc->spread_tile[d] : dspread[d];
        ti[d] = desc->interp_tile[d] > 0 ? desc->interp_tile[d] : dinterp[d];
    }
    p->coil_group = desc->coil_group > 0 ? desc->coil_group : 8;
    if (p->coil_group != 1 && p->coil_group != 2 && p->coil_group != 4 && p->coil_group != 8) {
        delete p;
        return fail(GBN_ERR_ARG, "coil_group must be 1, 2, 4 or 8");
    }
    p->interp_coil_group = desc->interp_coil_group;
    if (p->interp_coil_group != 0 && p->interp_coil_group != 1 && p->interp_coil_group != 2 &&
        p->interp_coil_group != 4 && p->interp_coil_group != 8) {
        delete p;
        return fail(GBN_ERR_ARG, "interp_coil_group must be 0, 1, 2, 4 or 8");
    }
    if (desc->interp_staging != 0 && desc->interp_staging != 1) {
        delete p;
        return fail(GBN_ERR_ARG, "interp_staging must be 0 or 1");
    }
    p->interp_staging = desc->interp_staging;
    if (desc->interp_variant < 0 || desc->interp_variant > 2) {
        delete p;
        return fail(GBN_ERR_ARG, "interp_variant must be 0, 1 or 2");
    }
    p->interp_variant = desc->interp_variant;
    if (desc->spread_variant < 0 || desc->spread_variant > 3) {
        delete p;
        return fail(GBN_ERR_ARG, "spread_variant must be 0, 1, 2 or 3");
    }
    p->spread_variant = desc->spread_variant;
    if (desc->fft_variant < 0 || desc->fft_variant > 2) {
        delete p;
        return fail(GBN_ERR_ARG, "fft_variant must be 0, 1 or 2");
    }
    p->fft_variant = desc->fft_variant;
    p->dense_min = desc->dense_tile_samples > 0 ? desc->dense_tile_samples
                                                : (desc->dense_tile_samples < 0 ? 0 : kDenseDefault);
    p->threads = desc->threads > 0 ? desc->threads : 256;
    p->interp_threads = desc->interp_threads > 0 ? desc->interp_threads : (p->dim == 2 ? 512 : 256);
    for (int t : {p->threads, p->interp_threads}) {
        if (t != 128 && t != 256 && t != 512) {
            delete p;
            return fail(GBN_ERR_ARG, "threads must be 128, 256 or 512");
        }
    }
    // 2-D with 4 or 8 coils per block: the register-tile spread kernel, whose tile is
    // (4 rows x warps) x (4 columns x 32/coils) cells, unless the caller chose a tile.
    // Measured on GB300 (8 coils, 512^2 radial): 128-thread blocks, 128-sample work items.
    bool reg_spread = false;
    const int cg_eff = std::min(p->coil_group, pow2_floor(std::max(1, (int)desc->n_coil)));
    if (p->dim == 2 && desc->spread_tile[0] <= 0 && desc->spread_tile[1] <= 0 && cg_eff >= 4) {
        if (desc->threads <= 0) p->threads = 128;
        if (p->threads <= 256) {
            ts[0] = 4 * (p->threads / 32);
            ts[1] = 4 * (32 / cg_eff);
            reg_spread = true;
        }
    }
    // 3-D with 8 coils per block, unless the caller chose a tile: the tensor-core kernel on
    // 4 x 8 x 16 tiles (variant 0 or 3), or the cube kernel on 8^3-cell tiles (2 x 2 x 2 cubes
    // of 4^3, variant 2), with 2048-sample work items.  Measured on GB300 (8 coils, 2.56 M
    // centre-out radial samples, 256^3 grid), with the dense centre tiles on the compensated
    // cubes: 7.8 ms (tensor cores), 11.3 ms (cubes), 13.9 ms (the warp rows' best tiling).
    // Otherwise (4 coils per block, or warp rows) the register rows: (x, y) rows of 4 per
    // warp, tile (TX, TY, 4 x 32/coils), TX*TY = 4 x warps.
    const bool tile_given = desc->spread_tile[0] > 0 || desc->spread_tile[1] > 0 || desc->spread_tile[2] > 0;
    if (p->dim == 2 && !tile_given && cg_eff == 8 && p->spread_variant == 3) {
        ts[0] = 8;  // the 2-D tensor-core kernel's tile: 128 cells, one TMEM lane each
        ts[1] = 16;
    } else if (p->dim == 3 && !tile_given && cg_eff == 8 && (p->spread_variant == 3 || p->spread_variant == 0)) {
        ts[0] = 4;  // the tensor-core kernel's tile: (y, z) = 128 cells, one TMEM lane each
        ts[1] = 8;
        ts[2] = 16;
        p->spread_variant = 3;
    } else if (p->dim == 3 && !tile_given && cg_eff == 8 && p->spread_variant == 2) {
        ts[0] = ts[1] = ts[2] = 8;
    } else if (p->dim == 3 && !tile_given && cg_eff >= 4 && p->threads <= 256) {
        const int rows = 4 * (p->threads / 32);
        ts[1] = rows >= 32 ? 8 : 4;
        ts[0] = rows / ts[1];
        ts[2] = 4 * (32 / cg_eff);
        reg_spread = true;
    }
    // the cube and tensor-core kernels keep a ring of batches full: long work items (the 3-D
    // tensor-core spread and interp share the work items; measured on the 3-D radial
    // workload: interp 3.75 ms at 4096 samples against 3.93 at 2048, spread even)
    const bool cube = cg_eff == 8 && ((p->dim == 3 && p->spread_variant == 2) || p->spread_variant == 3);
    const bool mma3 = cube && p->dim == 3 && p->spread_variant == 3;
    p->max_sub = desc->max_subproblem > 0 ? desc->max_subproblem
                                          : (mma3 ? 4096 : (cube ? 2048 : (reg_spread && p->dim == 2 ? 128 : 256)));
    make_geom(p, ts, p->gs);
    make_geom(p, ti, p->gi);

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&p->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) {
        delete p;
        return fail(GBN_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }

    auto bail = [&](int code) {
        gbn_plan_destroy(p);
        return code;
    };
    const size_t grid_bytes = sizeof(float2) * (size_t)p->G * (size_t)p->n_inst;
    e = cudaMalloc((void **)&p->grid, grid_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        p->grid = nullptr;
        return bail(fail(GBN_ERR_ALLOC, "grid allocation of " + std::to_string(grid_bytes) + " bytes failed"));
    }
    p->device_bytes += grid_bytes;
    for (int d = 0; d < 3; ++d) {
        e = cudaMalloc((void **)&p->tab[d], sizeof(float) * p->m[d]);
        if (e != cudaSuccess) {
            cudaGetLastError();
            p->tab[d] = nullptr;
            return bail(fail(GBN_ERR_ALLOC, "table allocation failed"));
        }
        p->device_bytes += sizeof(float) * p->m[d];
    }
    // word 0: kernel status bits; words 1, 2: dense spread subproblems and split spread
    // tiles (counted by set_points); words 3, 4: the cursors of the split-tile and
    // dense-subproblem lists
    e = cudaMalloc((void **)&p->kstatus, 8 * sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaGetLastError();
        p->kstatus = nullptr;
        return bail(fail(GBN_ERR_ALLOC, "status word allocation failed"));
    }
    e = cudaMemset(p->kstatus, 0, 8 * sizeof(uint32_t));
    if (e == cudaSuccess) e = launch_build_tables(p->dim, p->m, p->nf, p->tau, p->tab[0], p->tab[1], p->tab[2], 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return bail(fail(GBN_ERR_CUDA, std::string("table build: ") + cudaGetErrorString(e)));

    int n[3] = {p->nf[0], p->nf[1], p->nf[2]};
    if (p->G * p->n_inst >= ((int64_t)1 << 62) || p->n_inst > 0x7FFFFFFF)
        return bail(fail(GBN_ERR_CAPACITY, "batch too large for cuFFT"));
    cufftResult r = cufftPlanMany(&p->fft, p->dim, n, nullptr, 1, (int)p->G, nullptr, 1, (int)p->G, CUFFT_C2C,
                                  (int)p->n_inst);
    if (r != CUFFT_SUCCESS)
        return bail(fail(GBN_ERR_CUFFT, "cufftPlanMany failed, cufftResult " + std::to_string((int)r)));
    p->fft_ok = true;
    size_t ws = 0;
    if (cufftGetSize(p->fft, &ws) == CUFFT_SUCCESS) p->device_bytes += ws;
    if (fft_band_wanted(p)) {
        const int st = make_fft_band(p);
        if (st != GBN_OK) {
            if (p->fft_variant == 2) return bail(st);  // asked for: its failure is the plan's
            drop_fft_band(p);  // the library's choice: the full transform instead
        }
    }
    *out = p;
    return GBN_OK;
}

}  // namespace

// =====================================================================================
extern "C" {

int gbn_version(void) { return 100; }

const char *gbn_status_string(int status) {
    switch (status) {
        case GBN_OK: return "ok";
        case GBN_ERR_ARG: return "invalid argument";
        case GBN_ERR_ALLOC: return "allocation failed";
        case GBN_ERR_CUDA: return "CUDA error";
        case GBN_ERR_CUFFT: return "cuFFT error";
        case GBN_ERR_STATE: return "invalid call order";
        case GBN_ERR_CAPACITY: return "size beyond a supported limit";
        case GBN_ERR_INTERNAL: return "internal error";
        case GBN_ERR_TIMEOUT: return "a kernel's bounded wait gave up";
        default: return "unknown status";
    }
}

int gbn_last_error(char *buf, int len) {
    if (!buf || len <= 0) return GBN_ERR_ARG;
    std::snprintf(buf, (size_t)len, "%s", g_last_error.c_str());
    return GBN_OK;
}

int gbn_grid_params(int dim, int ms, int mt, int mu, double eps, int max_nspread, int *nspread, int64_t nf[3],
                    double *tau) {
    if (!nspread || !nf || !tau) return fail(GBN_ERR_ARG, "null output pointer");
    return compute_params(dim, ms, mt, mu, eps, max_nspread, nspread, nf, tau);
}

int gbn_plan_create(const gbn_plan_desc *desc, gbn_plan **out) {
    try {
        return plan_create_impl(desc, out);
    } catch (...) {
        return fail(GBN_ERR_INTERNAL, "exception in gbn_plan_create");
    }
}

int gbn_plan_destroy(gbn_plan *p) {
    if (!p) return GBN_OK;
    if (p->fft_ok) cufftDestroy(p->fft);
    for (int i = 0; i < p->fft_n_planes; ++i) cufftDestroy(p->fft_planes[i]);
    if (p->fft_x_ok) cufftDestroy(p->fft_x);
    if (p->fft_work) cudaFree(p->fft_work);
    if (p->grid) cudaFree(p->grid);
    if (p->kstatus) cudaFree(p->kstatus);
    for (int d = 0; d < 3; ++d)
        if (p->tab[d]) cudaFree(p->tab[d]);
    DevBuf *bufs[] = {&p->traj_off_d, &p->grp_scale, &p->pts, &p->home_key, &p->home_keys_sorted,
                      &p->touch_count, &p->touch_off, &p->home_count, &p->iota, &p->home_idx, &p->home_pts,
                      &p->dup_keys, &p->dup_vals, &p->dup_keys_sorted, &p->dup_idx, &p->dup_pts,
                      &p->spread_count, &p->spread_tile_off, &p->home_tile_off, &p->nsub, &p->sub_off, &p->nsub_i, &p->sub_off_i,
                      &p->spread_subs, &p->interp_subs, &p->cub_tmp, &p->scratch, &p->stage_in,
                      &p->stage_out, &p->stage_w, &p->split_tiles, &p->dense_subs, &p->solve_ws, &p->dcf_ws};
    for (gbn_plan::SolveGraph &sg : p->solve_graph)
        if (sg.exec) cudaGraphExecDestroy(sg.exec);
    for (DevBuf *b : bufs) release(*b);
    delete p;
    return GBN_OK;
}

int gbn_plan_status(gbn_plan *p, gbn_stream_t stream) {
    if (!p) return fail(GBN_ERR_ARG, "null plan");
    const cudaStream_t s = (cudaStream_t)stream;
    uint32_t st = 0;
    GBN_CUDA(cudaStreamSynchronize(s));
    GBN_CUDA(cudaMemcpy(&st, p->kstatus, sizeof(st), cudaMemcpyDeviceToHost));
    if (st == 0) return GBN_OK;
    GBN_CUDA(cudaMemset(p->kstatus, 0, sizeof(uint32_t)));
    return fail(GBN_ERR_TIMEOUT, "status word " + std::to_string(st) +
                                     ": a bounded wait gave up (bit 2: an interp tensor copy, bit 4: the 3-D spread's "
                                     "batch ring)");
}

}  // extern "C"

namespace {
// the bounded-wait self-test kernel: an mbarrier armed for bytes no copy will deliver
__global__ void k_wait_selftest(uint32_t probes, uint32_t *status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    gbn::mbar_init(&bar, 1);
    gbn::fence_barrier_init();
    gbn::mbar_arrive_expect_tx(&bar, 16);
    if (!gbn::mbar_wait_bounded(&bar, 0, probes)) atomicOr(status, gbn::kStatusTmaTimeout);
}
}  // namespace

extern "C" {

int gbn_plan_check_wait_expiry(gbn_plan *p, uint32_t probes, gbn_stream_t stream) {
    if (!p) return fail(GBN_ERR_ARG, "null plan");
    if (probes < 1 || probes > 65536) return fail(GBN_ERR_ARG, "probes must be in 1 .. 65536");
    k_wait_selftest<<<1, 32, 0, (cudaStream_t)stream>>>(probes, p->kstatus);
    GBN_CUDA(cudaGetLastError());
    return GBN_OK;
}

int gbn_plan_get_info(const gbn_plan *p, gbn_plan_info *o) {
    if (!p || !o) return fail(GBN_ERR_ARG, "null argument");
    std::memset(o, 0, sizeof(*o));
    o->nspread = p->ns;
    for (int d = 0; d < 3; ++d) {
        o->nf[d] = p->nf[d];
        o->spread_tile[d] = p->gs.tile[d];
        o->interp_tile[d] = p->gi.tile[d];
    }
    o->tau = p->tau;
    o->n_samples = p->M;
    o->grid_cells = p->G;
    o->n_inst = p->n_inst;
    o->spread_subproblems = p->n_spread_sub;
    o->interp_subproblems = p->n_interp_sub;
    o->spread_entries = p->n_dup;
    o->coil_group = p->coil_group;
    o->threads = p->threads;
    o->interp_threads = p->interp_threads;
    o->max_subproblem = p->max_sub;
    o->interp_coil_group = interp_cg(p);
    o->dense_subproblems = p->n_dense_sub;
    o->spread_kernels = p->spread_kernels;
    o->split_tiles = p->n_split;
    o->spread_variant = spread_path_kind(p->gs, spread_cg(p), p->spread_variant, p->threads);
    o->interp_variant = interp_on_tensor_cores(p) ? 2 : 1;
    o->fft_variant = p->fft_band ? 2 : 1;
    o->device_bytes = (int64_t)p->device_bytes;
    return GBN_OK;
}

int gbn_set_points(gbn_plan *p, int coord_dtype, const void *x, const void *y, const void *z,
                   const int64_t *traj_offsets, gbn_stream_t stream) {
    try {
        return set_points_impl(p, coord_dtype, x, y, z, traj_offsets, (cudaStream_t)stream);
    } catch (...) {
        return fail(GBN_ERR_INTERNAL, "exception in gbn_set_points");
    }
}

void *gbn_plan_grid(gbn_plan *p) { return p ? (void *)p->grid : nullptr; }

int gbn_spread(gbn_plan *p, const void *c, gbn_layout L, void *grid, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if ((!c && p->M > 0) || !grid) return fail(GBN_ERR_ARG, "null buffer");
    return run_spread(p, c, L, nullptr, (float2 *)grid, (cudaStream_t)stream);
}

int gbn_interp(gbn_plan *p, const void *grid, void *c, gbn_layout L, const float *weight, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if ((!c && p->M > 0) || !grid) return fail(GBN_ERR_ARG, "null buffer");
    return run_interp(p, (const float2 *)grid, c, L, weight, (cudaStream_t)stream);
}

int gbn_fft(gbn_plan *p, void *grid, int direction, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, false));
    if (!grid) return fail(GBN_ERR_ARG, "null buffer");
    return fft_exec(p, (float2 *)grid, direction, (cudaStream_t)stream);
}

int gbn_fft_band(gbn_plan *p, void *grid, int direction, int band, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, false));
    if (!grid) return fail(GBN_ERR_ARG, "null buffer");
    if (band != GBN_BAND_INPUT && band != GBN_BAND_OUTPUT)
        return fail(GBN_ERR_ARG, "band must be GBN_BAND_INPUT or GBN_BAND_OUTPUT");
    return fft_band_exec(p, (float2 *)grid, direction, band, (cudaStream_t)stream);
}

int gbn_pad_deapod(gbn_plan *p, const void *img, gbn_layout L, void *grid, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, false));
    if (!img || !grid) return fail(GBN_ERR_ARG, "null buffer");
    GBN_CUDA(launch_pad(deapod_args(p, false), (const float2 *)img, L, (float2 *)grid, (cudaStream_t)stream));
    return GBN_OK;
}

int gbn_crop_deapod(gbn_plan *p, const void *grid, void *img, gbn_layout L, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if (!img || !grid) return fail(GBN_ERR_ARG, "null buffer");
    GBN_CUDA(launch_crop(deapod_args(p, true), (const float2 *)grid, (float2 *)img, L, (cudaStream_t)stream));
    return GBN_OK;
}

int gbn_type1(gbn_plan *p, const void *c, gbn_layout cl, const float *weight, void *img, gbn_layout il,
              gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if ((!c && p->M > 0) || !img) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    GBN_TRY(run_spread(p, c, cl, weight, p->grid, s));
    GBN_TRY(fft_band_exec(p, p->grid, dir_type1(p), GBN_BAND_OUTPUT, s));
    GBN_CUDA(launch_crop(deapod_args(p, true), p->grid, (float2 *)img, il, s));
    return GBN_OK;
}

int gbn_type2(gbn_plan *p, const void *img, gbn_layout il, void *c, gbn_layout cl, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if ((!c && p->M > 0) || !img) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    GBN_CUDA(launch_pad(deapod_args(p, false), (const float2 *)img, il, p->grid, s));
    GBN_TRY(fft_band_exec(p, p->grid, dir_type2(p), GBN_BAND_INPUT, s));
    GBN_TRY(run_interp(p, p->grid, c, cl, nullptr, s));
    return GBN_OK;
}

int gbn_type21(gbn_plan *p, const void *img, gbn_layout il, void *out, gbn_layout ol, const float *dcf,
               gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if (!img || !out) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const gbn_layout sl = {0, 1, p->desc.n_coil};
    GBN_CUDA(launch_pad(deapod_args(p, false), (const float2 *)img, il, p->grid, s));
    GBN_TRY(fft_band_exec(p, p->grid, dir_type2(p), GBN_BAND_INPUT, s));
    GBN_TRY(run_interp(p, p->grid, p->scratch.p, sl, dcf, s));
    GBN_TRY(run_spread(p, p->scratch.p, sl, nullptr, p->grid, s));
    GBN_TRY(fft_band_exec(p, p->grid, dir_type1(p), GBN_BAND_OUTPUT, s));
    GBN_CUDA(launch_crop(deapod_args(p, true), p->grid, (float2 *)out, ol, s));
    return GBN_OK;
}

int gbn_sense_forward(gbn_plan *p, const void *x, gbn_layout xl, const void *sens, gbn_layout sl, void *kdata,
                      gbn_layout kl, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if (!x || !sens || (!kdata && p->M > 0)) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    GBN_CUDA(launch_pad_sense(deapod_args(p, false), (const float2 *)x, xl, (const float2 *)sens, sl, p->grid, s));
    GBN_TRY(fft_band_exec(p, p->grid, dir_type2(p), GBN_BAND_INPUT, s));
    GBN_TRY(run_interp(p, p->grid, kdata, kl, nullptr, s));
    return GBN_OK;
}

int gbn_sense_adjoint(gbn_plan *p, const void *kdata, gbn_layout kl, const float *dcf, const void *sens,
                      gbn_layout sl, void *x, gbn_layout xl, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if (!x || !sens || (!kdata && p->M > 0)) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    GBN_TRY(run_spread(p, kdata, kl, dcf, p->grid, s));
    GBN_TRY(fft_band_exec(p, p->grid, dir_type1(p), GBN_BAND_OUTPUT, s));
    GBN_CUDA(launch_crop_sense(deapod_args(p, true), p->grid, (const float2 *)sens, sl, (float2 *)x, xl, s));
    return GBN_OK;
}

int gbn_sense_normal(gbn_plan *p, const void *x, gbn_layout xl, const void *sens, gbn_layout sl,
                     const float *dcf, void *x_out, gbn_layout ol, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if (!x || !sens || !x_out) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const gbn_layout scl = {0, 1, p->desc.n_coil};
    GBN_CUDA(launch_pad_sense(deapod_args(p, false), (const float2 *)x, xl, (const float2 *)sens, sl, p->grid, s));
    GBN_TRY(fft_band_exec(p, p->grid, dir_type2(p), GBN_BAND_INPUT, s));
    GBN_TRY(run_interp(p, p->grid, p->scratch.p, scl, dcf, s));
    GBN_TRY(run_spread(p, p->scratch.p, scl, nullptr, p->grid, s));
    GBN_TRY(fft_band_exec(p, p->grid, dir_type1(p), GBN_BAND_OUTPUT, s));
    GBN_CUDA(launch_crop_sense(deapod_args(p, true), p->grid, (const float2 *)sens, sl, (float2 *)x_out, ol, s));
    return GBN_OK;
}

int gbn_interp_grad_coords(gbn_plan *p, const void *grid, const void *grad_c, gbn_layout cl, float *grad_xyz,
                           gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if (!grid || ((!grad_c || !grad_xyz) && p->M > 0)) return fail(GBN_ERR_ARG, "null buffer");
    if (p->M == 0) return GBN_OK;
    cudaStream_t s = (cudaStream_t)stream;
    GBN_CUDA(cudaMemsetAsync(grad_xyz, 0, sizeof(float) * (size_t)p->M * p->dim, s));
    GradArgs a;
    a.g = p->gi;
    a.subs = p->interp_subs.as<int4>();
    a.pts = p->home_pts.as<float4>();
    a.idx = p->home_idx.as<uint32_t>();
    a.grid = (const float2 *)grid;
    a.gc = (const float2 *)grad_c;
    a.c_elem = cl.elem_stride;
    a.c_coil = cl.coil_stride;
    a.out = grad_xyz;
    a.scale = (float)p->desc.df;
    const int cg = interp_cg(p);
    GBN_CUDA(launch_interp_grad(a, p->n_interp_sub, cg, p->interp_threads, s));
    return GBN_OK;
}

int gbn_graph_capture_normal(gbn_plan *p, const void *x, gbn_layout xl, const void *sens, gbn_layout sl,
                             const float *dcf, void *x_out, gbn_layout ol, gbn_graph **out) {
    GBN_TRY(check_plan(p, true));
    if (!out) return fail(GBN_ERR_ARG, "null output");
    *out = nullptr;
    cudaStream_t s;
    GBN_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    gbn_graph *g = new (std::nothrow) gbn_graph();
    if (!g) {
        cudaStreamDestroy(s);
        return fail(GBN_ERR_ALLOC, "host allocation failed");
    }
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    int st = GBN_OK;
    if (e == cudaSuccess) {
        st = sens ? gbn_sense_normal(p, x, xl, sens, sl, dcf, x_out, ol, (gbn_stream_t)s)
                  : gbn_type21(p, x, xl, x_out, ol, dcf, (gbn_stream_t)s);
        cudaGraph_t graph = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(s, &graph);
        if (e2 == cudaSuccess && st == GBN_OK) {
            g->graph = graph;
            e = cudaGraphInstantiate(&g->exec, graph, 0);
        } else {
            if (graph) cudaGraphDestroy(graph);
            if (st == GBN_OK) e = e2;
        }
    }
    cudaStreamDestroy(s);
    if (st != GBN_OK || e != cudaSuccess) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        if (g->graph) cudaGraphDestroy(g->graph);
        delete g;
        cudaGetLastError();
        return st != GBN_OK ? st : fail(GBN_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    *out = g;
    return GBN_OK;
}

int gbn_graph_launch(gbn_graph *g, gbn_stream_t stream) {
    if (!g || !g->exec) return fail(GBN_ERR_ARG, "null graph");
    GBN_CUDA(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    return GBN_OK;
}

int gbn_graph_destroy(gbn_graph *g) {
    if (!g) return GBN_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return GBN_OK;
}

}  // extern "C"

// ---- solvers ------------------------------------------------------------------------------
namespace {

constexpr size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Vectors of a solve: x is one image per trajectory group, (n_traj, pixels) with sens, or
// the plan's coil-last images (n_traj, pixels, n_coil) without; contiguous complex64.
struct SolveVecs {
    int64_t n = 0;            // complex elements per vector
    gbn_layout layout{};      // of every vector, for the normal operator
    HaarGeom h{};
    SolveState *st = nullptr;
    double *partial = nullptr, *norms = nullptr;
    float2 *v[5] = {};
    int cap = 0;
};

int solve_setup(gbn_plan *p, const void *sens, int n_iter, int level, SolveVecs &sv) {
    const int64_t P = (int64_t)p->m[0] * p->m[1] * p->m[2];
    const int64_t inner = sens ? 1 : p->desc.n_coil;
    sv.n = P * inner * p->desc.n_traj;
    sv.layout = sens ? gbn_layout{P, 0, 1} : gbn_layout{P * inner, 1, inner};
    const int32_t shape[3] = {p->m[0], p->m[1], p->m[2]};
    if (level >= 0) GBN_TRY(haar_geom(p->dim, shape, level, p->desc.n_traj, inner, sv.h));
    sv.cap = 64;
    while (sv.cap < n_iter) sv.cap *= 2;
    const size_t vec = align256(sizeof(float2) * (size_t)sv.n);
    const size_t off_partial = align256(sizeof(SolveState));
    const size_t off_norms = off_partial + align256(sizeof(double) * kRedBlocks);
    const size_t off_vec = off_norms + align256(sizeof(double) * (size_t)sv.cap);
    GBN_TRY(ensure(p, p->solve_ws, off_vec + 5 * vec));
    char *base = p->solve_ws.as<char>();
    sv.st = (SolveState *)base;
    sv.partial = (double *)(base + off_partial);
    sv.norms = (double *)(base + off_norms);
    for (int i = 0; i < 5; ++i) sv.v[i] = (float2 *)(base + off_vec + i * vec);
    return GBN_OK;
}

int solve_normal(gbn_plan *p, const SolveVecs &sv, const void *sens, gbn_layout sl, const float *dcf,
                 const float2 *in, float2 *out, cudaStream_t s) {
    return sens ? gbn_sense_normal(p, in, sv.layout, sens, sl, dcf, out, sv.layout, (gbn_stream_t)s)
                : gbn_type21(p, in, sv.layout, out, sv.layout, dcf, (gbn_stream_t)s);
}

// One solver iteration as a callable; with a graph it is captured once per (kind, operator
// inputs, workspace, points) and replayed.
template <typename F>
int run_iterations(gbn_plan *p, int kind, const void *sens, gbn_layout sl, const float *dcf, const SolveVecs &sv,
                   int level, float step, float th, int n, bool use_graph, cudaStream_t s, F &&iteration) {
    if (n <= 0) return GBN_OK;
    if (!use_graph) {
        for (int i = 0; i < n; ++i) GBN_TRY(iteration(s));
        return GBN_OK;
    }
    gbn_plan::SolveGraph &g = p->solve_graph[kind];
    const bool hit = g.exec && g.sens == sens && g.sl.traj_stride == sl.traj_stride &&
                     g.sl.coil_stride == sl.coil_stride && g.sl.elem_stride == sl.elem_stride && g.dcf == dcf &&
                     g.ws == p->solve_ws.p && g.gen == p->points_gen && g.cap == sv.cap && g.level == level &&
                     g.step == step && g.th == th;
    if (!hit) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = gbn_plan::SolveGraph{};
        cudaStream_t cs;
        GBN_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        int st = GBN_OK;
        cudaGraph_t graph = nullptr;
        if (e == cudaSuccess) {
            st = iteration(cs);
            cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
            if (st == GBN_OK && e2 == cudaSuccess) e = cudaGraphInstantiate(&g.exec, graph, 0);
            else if (st == GBN_OK) e = e2;
            if (graph) cudaGraphDestroy(graph);
        }
        cudaStreamDestroy(cs);
        if (st != GBN_OK || e != cudaSuccess) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g = gbn_plan::SolveGraph{};
            cudaGetLastError();
            return st != GBN_OK ? st : fail(GBN_ERR_CUDA, std::string("solver graph capture: ") + cudaGetErrorString(e));
        }
        g.sens = sens;
        g.sl = sl;
        g.dcf = dcf;
        g.ws = p->solve_ws.p;
        g.gen = p->points_gen;
        g.cap = sv.cap;
        g.level = level;
        g.step = step;
        g.th = th;
    }
    for (int i = 0; i < n; ++i) GBN_CUDA(cudaGraphLaunch(g.exec, s));
    return GBN_OK;
}

int check_solve(const gbn_plan *p, const void *rhs, const void *x, int n_iter) {
    GBN_TRY(check_plan(p, true));
    if (!rhs || !x) return fail(GBN_ERR_ARG, "null buffer");
    if (n_iter < 1) return fail(GBN_ERR_ARG, "n_iter must be >= 1");
    return GBN_OK;
}

}  // namespace

extern "C" {

int gbn_cg_sense(gbn_plan *p, const void *sens, gbn_layout sl, const float *dcf, const void *rhs, void *x,
                 int32_t n_iter, double *res_norms, int32_t flags, gbn_stream_t stream) {
    GBN_TRY(check_solve(p, rhs, x, n_iter));
    cudaStream_t s = (cudaStream_t)stream;
    SolveVecs sv;
    GBN_TRY(solve_setup(p, sens, n_iter, -1, sv));
    float2 *xv = sv.v[0], *r = sv.v[1], *pv = sv.v[2], *q = sv.v[3];
    const size_t bytes = sizeof(float2) * (size_t)sv.n;
    GBN_CUDA(cudaMemsetAsync(sv.st, 0, sizeof(SolveState), s));
    if (flags & GBN_SOLVE_X0) {
        GBN_CUDA(cudaMemcpyAsync(xv, x, bytes, cudaMemcpyDeviceToDevice, s));
        GBN_TRY(solve_normal(p, sv, sens, sl, dcf, xv, q, s));
        GBN_CUDA(launch_cg_start((const float2 *)rhs, q, r, pv, sv.n, sv.partial, sv.st, s));
    } else {
        GBN_CUDA(cudaMemsetAsync(xv, 0, bytes, s));
        GBN_CUDA(launch_cg_start((const float2 *)rhs, nullptr, r, pv, sv.n, sv.partial, sv.st, s));
    }
    auto iteration = [&](cudaStream_t cs) -> int {
        GBN_TRY(solve_normal(p, sv, sens, sl, dcf, pv, q, cs));
        GBN_CUDA(launch_cg_alpha(pv, q, sv.n, sv.partial, sv.st, cs));
        GBN_CUDA(launch_cg_update(xv, r, pv, q, sv.n, sv.partial, sv.st, sv.norms, sv.cap, cs));
        GBN_CUDA(launch_cg_direction(r, pv, sv.n, sv.st, cs));
        return GBN_OK;
    };
    GBN_TRY(run_iterations(p, 0, sens, sl, dcf, sv, -1, 0.f, 0.f, n_iter, !(flags & GBN_SOLVE_NO_GRAPH), s,
                           iteration));
    GBN_CUDA(cudaMemcpyAsync(x, xv, bytes, cudaMemcpyDeviceToDevice, s));
    if (res_norms)
        GBN_CUDA(cudaMemcpyAsync(res_norms, sv.norms, sizeof(double) * n_iter, cudaMemcpyDeviceToDevice, s));
    return GBN_OK;
}

int gbn_dcf_pipe_menon(gbn_plan *p, int32_t n_iter, float *dcf, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if (n_iter < 1) return fail(GBN_ERR_ARG, "n_iter must be >= 1");
    if (p->desc.n_coil != 1) return fail(GBN_ERR_ARG, "density estimation takes a plan with n_coil == 1");
    if (p->M == 0) return GBN_OK;
    if (!dcf) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t w_bytes = align256(sizeof(float2) * (size_t)p->M);
    GBN_TRY(ensure(p, p->dcf_ws, w_bytes + sizeof(double) * kDcfPartials * (size_t)p->desc.n_traj));
    float2 *w = p->dcf_ws.as<float2>(), *cw = p->scratch.as<float2>();  // scratch: M x n_coil from set_points
    double *partial = (double *)(p->dcf_ws.as<char>() + w_bytes);
    const gbn_layout cl = {0, 1, 1};
    GBN_CUDA(launch_dcf_fill(w, p->M, s));
    for (int it = 0; it < n_iter; ++it) {
        GBN_TRY(run_spread(p, w, cl, nullptr, p->grid, s));
        GBN_TRY(run_interp(p, p->grid, cw, cl, nullptr, s));
        GBN_CUDA(launch_dcf_update(w, cw, p->M, s));
    }
    GBN_CUDA(launch_dcf_finish(w, p->traj_off_d.as<int64_t>(), p->desc.n_traj, partial, dcf, s));
    return GBN_OK;
}

int gbn_ista_haar(gbn_plan *p, const void *sens, gbn_layout sl, const float *dcf, const void *rhs, void *x,
                  int32_t n_iter, float step, float th, int32_t level, int32_t flags, gbn_stream_t stream) {
    GBN_TRY(check_solve(p, rhs, x, n_iter));
    if (!std::isfinite(step) || !(th >= 0.f) || !std::isfinite(th))
        return fail(GBN_ERR_ARG, "step must be finite and th finite and >= 0");
    if (level < 0) return fail(GBN_ERR_ARG, "level must be >= 0");
    cudaStream_t s = (cudaStream_t)stream;
    SolveVecs sv;
    GBN_TRY(solve_setup(p, sens, n_iter, level, sv));
    const size_t bytes = sizeof(float2) * (size_t)sv.n;
    const bool fista = (flags & GBN_SOLVE_FISTA) != 0;
    float2 *acc = sv.v[0], *xv = sv.v[1], *q = sv.v[2], *b = sv.v[3], *x_pre = sv.v[4];
    GBN_CUDA(cudaMemsetAsync(sv.st, 0, sizeof(SolveState), s));
    GBN_CUDA(cudaMemcpyAsync(b, rhs, bytes, cudaMemcpyDeviceToDevice, s));
    HaarStepArgs a{};
    a.h = sv.h;
    a.acc = acc;
    a.rhs = b;
    a.step = step;
    a.th = th;
    a.st = sv.st;
    if (fista) {
        // y (the normal operator's input) lives in xv; x_pre carries x between iterations
        GBN_CUDA(launch_fista_start(b, step, xv, acc, x_pre, sv.n, sv.st, s));
        a.q = q;
        a.x_pre = x_pre;
        a.y = xv;
    } else {
        // IST_32: x_acc = step * rhs, x = prox(x_acc); then (normal, update + prox) n_iter - 1
        // times: the reference's last normal-operator call only feeds an x_acc it never uses
        GBN_CUDA(launch_scale(b, step, acc, sv.n, s));
        a.x_out = xv;
        GBN_CUDA(launch_haar_step(a, false, s));
        a.q = q;
    }
    auto iteration = [&](cudaStream_t cs) -> int {
        GBN_TRY(solve_normal(p, sv, sens, sl, dcf, xv, q, cs));
        GBN_CUDA(launch_haar_step(a, fista, cs));
        return GBN_OK;
    };
    GBN_TRY(run_iterations(p, fista ? 2 : 1, sens, sl, dcf, sv, level, step, th, fista ? n_iter : n_iter - 1,
                           !(flags & GBN_SOLVE_NO_GRAPH), s, iteration));
    GBN_CUDA(cudaMemcpyAsync(x, fista ? x_pre : xv, bytes, cudaMemcpyDeviceToDevice, s));
    return GBN_OK;
}

// ---- host-buffer entry points -----------------------------------------------------------
static int64_t image_elems(const gbn_plan *p) {
    return (int64_t)p->m[0] * p->m[1] * p->m[2] * p->desc.n_coil * p->desc.n_traj;
}
static gbn_layout host_img_layout(const gbn_plan *p) {
    const int64_t P = (int64_t)p->m[0] * p->m[1] * p->m[2];
    return gbn_layout{P * p->desc.n_coil, 1, p->desc.n_coil};
}
static gbn_layout host_sample_layout(const gbn_plan *p) { return gbn_layout{0, 1, p->desc.n_coil}; }

// Device address of a pinned (page-locked, mapped) host buffer, or null for pageable
// memory.  Kernels given it read or write the host memory directly over the host link, so
// the transfer overlaps the kernel instead of preceding or following it.
static void *mapped_host(const void *h) {
    if (!h) return nullptr;
    void *d = nullptr;
    if (cudaHostGetDevicePointer(&d, const_cast<void *>(h), 0) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return d;
}

int gbn_type1_host(gbn_plan *p, const void *h_c, void *h_img, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if ((!h_c && p->M > 0) || !h_img) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t cb = sizeof(float2) * (size_t)p->M * p->desc.n_coil, ib = sizeof(float2) * image_elems(p);
    // the spread gathers each sample several times (once per tile its stencil reaches):
    // the samples are copied in bulk; a pinned output image is written by the crop directly
    GBN_TRY(ensure(p, p->stage_in, cb));
    GBN_CUDA(cudaMemcpyAsync(p->stage_in.p, h_c, cb, cudaMemcpyHostToDevice, s));
    if (void *d_img = mapped_host(h_img)) {
        GBN_TRY(gbn_type1(p, p->stage_in.p, host_sample_layout(p), nullptr, d_img, host_img_layout(p), stream));
    } else {
        GBN_TRY(ensure(p, p->stage_out, ib));
        GBN_TRY(gbn_type1(p, p->stage_in.p, host_sample_layout(p), nullptr, p->stage_out.p, host_img_layout(p),
                          stream));
        GBN_CUDA(cudaMemcpyAsync(h_img, p->stage_out.p, ib, cudaMemcpyDeviceToHost, s));
    }
    GBN_CUDA(cudaStreamSynchronize(s));
    return GBN_OK;
}

int gbn_type2_host(gbn_plan *p, const void *h_img, void *h_c, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if ((!h_c && p->M > 0) || !h_img) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t cb = sizeof(float2) * (size_t)p->M * p->desc.n_coil, ib = sizeof(float2) * image_elems(p);
    // pinned buffers: the pad reads the image and the interp writes the samples directly --
    // except the tensor-core interp, which zeroes its output and adds per-tile partials with
    // atomics: it writes a device buffer that is copied back in bulk
    const void *src = mapped_host(h_img);
    void *dst = p->M > 0 && !interp_on_tensor_cores(p) ? mapped_host(h_c) : nullptr;
    if (!src) {
        GBN_TRY(ensure(p, p->stage_in, ib));
        GBN_CUDA(cudaMemcpyAsync(p->stage_in.p, h_img, ib, cudaMemcpyHostToDevice, s));
        src = p->stage_in.p;
    }
    if (!dst) {
        GBN_TRY(ensure(p, p->stage_out, cb));
        GBN_TRY(gbn_type2(p, src, host_img_layout(p), p->stage_out.p, host_sample_layout(p), stream));
        GBN_CUDA(cudaMemcpyAsync(h_c, p->stage_out.p, cb, cudaMemcpyDeviceToHost, s));
    } else {
        GBN_TRY(gbn_type2(p, src, host_img_layout(p), dst, host_sample_layout(p), stream));
    }
    GBN_CUDA(cudaStreamSynchronize(s));
    return GBN_OK;
}

int gbn_type21_host(gbn_plan *p, const void *h_img, void *h_out, const float *h_dcf, gbn_stream_t stream) {
    GBN_TRY(check_plan(p, true));
    if (!h_out || !h_img) return fail(GBN_ERR_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t ib = sizeof(float2) * image_elems(p);
    GBN_TRY(ensure(p, p->stage_in, ib));
    GBN_TRY(ensure(p, p->stage_out, ib));
    const float *dcf = nullptr;
    if (h_dcf) {
        GBN_TRY(ensure(p, p->stage_w, sizeof(float) * (size_t)p->M));
        GBN_CUDA(cudaMemcpyAsync(p->stage_w.p, h_dcf, sizeof(float) * (size_t)p->M, cudaMemcpyHostToDevice, s));
        dcf = p->stage_w.as<float>();
    }
    // pinned buffers: the pad reads and the crop writes them directly
    const void *src = mapped_host(h_img);
    void *dst = mapped_host(h_out);
    if (!src) {
        GBN_CUDA(cudaMemcpyAsync(p->stage_in.p, h_img, ib, cudaMemcpyHostToDevice, s));
        src = p->stage_in.p;
    }
    GBN_TRY(gbn_type21(p, src, host_img_layout(p), dst ? dst : p->stage_out.p, host_img_layout(p), dcf, stream));
    if (!dst) GBN_CUDA(cudaMemcpyAsync(h_out, p->stage_out.p, ib, cudaMemcpyDeviceToHost, s));
    GBN_CUDA(cudaStreamSynchronize(s));
    return GBN_OK;
}

// ---- one-shot reference-signature calls ---------------------------------------------------
static int one_shot(int dim, int kind, const double *x, const double *y, const double *z, const void *in,
                    int64_t M, int32_t ntrail, int32_t ms, int32_t mt, int32_t mu, const double *dcf, double df,
                    double eps, int32_t iflag, void *out) {
    if (M < 0 || ntrail < 1 || !x || !in || !out) return fail(GBN_ERR_ARG, "bad argument");
    if ((dim > 1 && !y) || (dim > 2 && !z)) return fail(GBN_ERR_ARG, "null coordinate");
    gbn_plan_desc d;
    std::memset(&d, 0, sizeof(d));
    d.dim = dim;
    d.ms = ms;
    d.mt = dim > 1 ? mt : 1;
    d.mu = dim > 2 ? mu : 1;
    d.eps = eps;
    d.max_nspread = dim == 3 ? 6 : 0;
    d.iflag = iflag;
    d.df = df;
    d.n_coil = ntrail;
    d.n_traj = 1;
    gbn_plan *p = nullptr;
    GBN_TRY(gbn_plan_create(&d, &p));
    cudaStream_t s = nullptr;
    double *dc[3] = {nullptr, nullptr, nullptr};
    float *dw = nullptr;
    int st = GBN_OK;
    const double *hc[3] = {x, y, z};
    auto cleanup = [&]() {
        for (int k = 0; k < 3; ++k)
            if (dc[k]) cudaFree(dc[k]);
        if (dw) cudaFree(dw);
        if (s) cudaStreamDestroy(s);
        gbn_plan_destroy(p);
    };
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        s = nullptr;
        cleanup();
        return fail(GBN_ERR_CUDA, "stream creation failed");
    }
    for (int k = 0; k < dim; ++k) {
        if (cudaMalloc(&dc[k], sizeof(double) * (size_t)std::max<int64_t>(M, 1)) != cudaSuccess ||
            cudaMemcpyAsync(dc[k], hc[k], sizeof(double) * (size_t)M, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            cudaGetLastError();
            cleanup();
            return fail(GBN_ERR_ALLOC, "coordinate upload failed");
        }
    }
    const int64_t off[2] = {0, M};
    st = gbn_set_points(p, GBN_COORD_F64, dc[0], dc[1], dc[2], off, (gbn_stream_t)s);
    if (st == GBN_OK && kind == 21 && dcf) {
        std::vector<float> w((size_t)M);
        for (int64_t i = 0; i < M; ++i) w[(size_t)i] = (float)dcf[i];
        st = gbn_type21_host(p, in, out, w.data(), (gbn_stream_t)s);
    } else if (st == GBN_OK) {
        if (kind == 1) st = gbn_type1_host(p, in, out, (gbn_stream_t)s);
        else if (kind == 2) st = gbn_type2_host(p, in, out, (gbn_stream_t)s);
        else st = gbn_type21_host(p, in, out, nullptr, (gbn_stream_t)s);
    }
    cleanup();
    return st;
}

int gbn_nufft2d1_gaussker(const double *x, const double *y, const void *c, int64_t M, int32_t ntrail, int32_t ms,
                          int32_t mt, double df, double eps, int32_t iflag, void *out) {
    return one_shot(2, 1, x, y, nullptr, c, M, ntrail, ms, mt, 1, nullptr, df, eps, iflag, out);
}
int gbn_nufft2d2_gaussker(const double *x, const double *y, const void *Fk, int64_t M, int32_t ntrail, int32_t ms,
                          int32_t mt, double df, double eps, int32_t iflag, void *out) {
    return one_shot(2, 2, x, y, nullptr, Fk, M, ntrail, ms, mt, 1, nullptr, df, eps, iflag, out);
}
int gbn_nufft2d21_gaussker(const double *x, const double *y, const void *Fk, int64_t M, int32_t ntrail,
                           int32_t ms, int32_t mt, double df, double eps, int32_t iflag, void *out) {
    return one_shot(2, 21, x, y, nullptr, Fk, M, ntrail, ms, mt, 1, nullptr, df, eps, iflag, out);
}
int gbn_nufft3d1_gaussker(const double *x, const double *y, const double *z, const void *c, int64_t M,
                          int32_t ntrail, int32_t ms, int32_t mt, int32_t mu, double df, double eps, int32_t iflag,
                          void *out) {
    return one_shot(3, 1, x, y, z, c, M, ntrail, ms, mt, mu, nullptr, df, eps, iflag, out);
}
int gbn_nufft3d2_gaussker(const double *x, const double *y, const double *z, const void *Fk, int64_t M,
                          int32_t ntrail, int32_t ms, int32_t mt, int32_t mu, double df, double eps, int32_t iflag,
                          void *out) {
    return one_shot(3, 2, x, y, z, Fk, M, ntrail, ms, mt, mu, nullptr, df, eps, iflag, out);
}
int gbn_nufft3d21_gaussker(const double *x, const double *y, const double *z, const void *Fk, int64_t M,
                           int32_t ntrail, int32_t ms, int32_t mt, int32_t mu, const double *dcf, double df,
                           double eps, int32_t iflag, void *out) {
    return one_shot(3, 21, x, y, z, Fk, M, ntrail, ms, mt, mu, dcf, df, eps, iflag, out);
}

}  // extern "C"
