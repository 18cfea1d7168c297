// Interp (type-2 gridding) and trajectory-gradient launchers.
//
// 2-D with at most 16 taps per dimension: k_interp2d_tma (persistent, windows staged by
// tensor copies; the caller supplies the tensor map) or k_interp2d (one block per
// subproblem, windows gathered by the threads).  3-D with at most 16 taps:
// k_interp3d_planes (4 or 8 coils per block, window streamed by x planes) or k_interp3d.
// Otherwise (1-D, wide stencils): k_interp (one thread per sample).
#include <algorithm>
#include <cstring>

#include "dispatch.cuh"
#include "grid2d_kernels.cuh"
#include "grid3d_kernels.cuh"
#include "interp2d_tma.cuh"
#include "interp3d_mma.cuh"

namespace gbn {

static bool use_2d_path(const Geom &g) { return g.dim == 2 && g.W <= 16; }

size_t interp3d_planes_smem(const Geom &g, int coil_group, int threads) {
    return interp3d_planes_smem_bytes(g, coil_group, threads > 256 ? 256 : threads);
}

// shared memory of the kernel launch_interp runs for this geometry, coil group and thread
// count (the 3-D kernel depends on all three)
size_t interp_smem_bytes(const Geom &g, int coil_group, int threads) {
    if (use_2d_path(g)) return interp2d_smem_bytes(g, coil_group);
    if (const size_t ps = interp3d_planes_smem_bytes(g, coil_group, threads > 256 ? 256 : threads)) return ps;
    size_t cells = 1;
    for (int d = 0; d < g.dim; ++d) cells *= (size_t)(g.tile[d] + g.W - 1);
    return cells * (size_t)coil_group * sizeof(float2);
}

static size_t grad_smem_bytes(const Geom &g, int coil_group) {
    size_t cells = 1;
    for (int d = 0; d < g.dim; ++d) cells *= (size_t)(g.tile[d] + g.W - 1);
    return cells * (size_t)coil_group * sizeof(float2);
}

bool interp3d_plane_box(const Geom &g, int coil_group, int &BY, int &BZ) {
    if (!interp3d_planes_smem_bytes(g, coil_group, 256)) return false;
    const PlaneBox pb = plane_box(g, coil_group);
    BY = pb.BY;
    BZ = pb.BZ;
    return true;
}

cudaError_t launch_interp3d_planes(const InterpArgs &a, int64_t n_sub, int coil_group, int threads,
                                   const CUtensorMap *map, uint32_t *status, cudaStream_t s) {
    if (n_sub == 0) return cudaSuccess;
    const int th = threads > 256 ? 256 : threads;
    const size_t smem = interp3d_planes_smem_bytes(a.g, coil_group, th);
    if (!smem) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)n_sub, (unsigned)((a.g.n_coil + coil_group - 1) / coil_group));
    const PlaneBox pb = plane_box(a.g, coil_group);
    CUtensorMap none;
    memset(&none, 0, sizeof(none));
    const int use_tma = map != nullptr && status != nullptr;
    cudaError_t err = cudaSuccess;
    GBN_DISPATCH_W(a.g.W, {
        auto kern = coil_group == 8 ? k_interp3d_planes<WT, 8> : k_interp3d_planes<WT, 4>;
        err = set_smem(kern, smem);
        if (err == cudaSuccess) {
            kern<<<grid, th, smem, s>>>(a, use_tma ? *map : none, pb, use_tma, status);
            err = cudaGetLastError();
        }
    });
    return err;
}

cudaError_t launch_interp(const InterpArgs &a, int64_t n_sub, int coil_group, int threads, cudaStream_t s) {
    if (n_sub == 0) return cudaSuccess;
    const size_t smem = interp_smem_bytes(a.g, coil_group, threads);
    const dim3 grid((unsigned)n_sub, (unsigned)((a.g.n_coil + coil_group - 1) / coil_group));
    cudaError_t err = cudaSuccess;
    if (use_2d_path(a.g)) {
        GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
            auto kern = k_interp2d<WT, CG>;
            err = set_smem(kern, smem);
            if (err == cudaSuccess) {
                kern<<<grid, threads, smem, s>>>(a);
                err = cudaGetLastError();
            }
        }));
        return err;
    }
    if (a.g.dim == 3 && a.g.W <= 16) {
        const int th = threads > 256 ? 256 : threads;
        if (interp3d_planes_smem_bytes(a.g, coil_group, th))  // 4 or 8 coils: stream plane by plane
            return launch_interp3d_planes(a, n_sub, coil_group, th, nullptr, nullptr, s);
        const size_t wsmem = interp3d_smem_bytes(a.g, coil_group);  // the whole staged window
        GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
            auto kern = k_interp3d<WT, CG>;
            err = set_smem(kern, wsmem);
            if (err == cudaSuccess) {
                kern<<<grid, th, wsmem, s>>>(a);
                err = cudaGetLastError();
            }
        }));
        return err;
    }
    GBN_DISPATCH_D(a.g.dim, GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
        auto kern = k_interp<D, WT, CG>;
        err = set_smem(kern, smem);
        if (err == cudaSuccess) {
            kern<<<grid, threads, smem, s>>>(a);
            err = cudaGetLastError();
        }
    })));
    return err;
}

// ---------------------------------------------------------------- tensor-core 3-D interp

bool interp_mma_applies(const Geom &gs, int coil_group) {
    return gs.dim == 3 && coil_group == 8 && grid3d_applies(gs) && gs.tile[0] == kMmaTX && gs.tile[1] == kMmaTY &&
           gs.tile[2] == kMmaTZ;
}

namespace {
// the output samples start from zero: the kernel adds every (sample, tile) partial
__global__ void k_zero_samples(float2 *c, int64_t M, int n_coil, int64_t c_elem, int64_t c_coil) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M * n_coil) return;
    const int64_t j = i / n_coil, coil = i - j * n_coil;
    c[j * c_elem + coil * c_coil] = make_float2(0.f, 0.f);
}
}  // namespace

cudaError_t launch_interp3d_mma(const MmaInterpArgs &a, int64_t n_sub, uint32_t *status, cudaStream_t s) {
    const int64_t n = a.M * a.g.n_coil;
    if (n == 0) return cudaSuccess;
    if (a.c_coil == 1 && a.c_elem == a.g.n_coil) {
        cudaError_t e = cudaMemsetAsync(a.c, 0, sizeof(float2) * (size_t)n, s);
        if (e != cudaSuccess) return e;
    } else {
        k_zero_samples<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a.c, a.M, a.g.n_coil, a.c_elem, a.c_coil);
    }
    if (n_sub == 0) return cudaGetLastError();
    const int n_cg = (a.g.n_coil + 7) / 8;
    // float4 atomics (two coils each) when the coils of a sample are adjacent and every
    // coil group starts on a 16-byte boundary (8-coil groups: an even element stride)
    // bit 0: two coils per atomicAdd(float4) into the samples; bit 1: the tile's grid values
    // loaded two z cells per 16-byte load (every such pair starts on a 16-byte boundary)
    const int vec = (a.c_coil == 1 && a.c_elem % 2 == 0 && (uintptr_t)a.c % 16 == 0 ? 1 : 0) |
                    ((uintptr_t)a.grid % 16 == 0 && a.g.nf[2] % 2 == 0 && a.g.G % 2 == 0 ? 2 : 0);
    cudaError_t err = cudaSuccess;
    GBN_DISPATCH_W(a.g.W, {
        auto kern = k_interp3d_mma<WT>;
        err = set_smem(kern, kImSmemBytes);
        if (err == cudaSuccess) {
            kern<<<(unsigned)(n_sub * n_cg), kImThreads, kImSmemBytes, s>>>(a, status, n_cg, vec);
            err = cudaGetLastError();
        }
    });
    return err;
}

// ---------------------------------------------------------------- TMA-staged 2-D interp

// Box of a staged window: BX >= WX rows and BY >= WY + 1 cells (even, since the window may
// start one cell into a row), smallest area such that the coil stride CS = BX * BY puts the
// CG coil runs of a half-warp's 8-byte loads on distinct banks: CS = 2 (mod 4) for 8 coils,
// 4 (mod 8) for 4, 8 (mod 16) for 2.
bool tma_window(const Geom &g, int cg, int64_t n_sub, TmaWin &t) {
    if (g.dim != 2 || g.W > 16 || (g.nf[1] & 1)) return false;
    const int WX = g.tile[0] + g.W - 1, WY = g.tile[1] + g.W - 1;
    const int mod = cg == 8 ? 4 : (cg == 4 ? 8 : (cg == 2 ? 16 : 1));
    const int want = cg == 8 ? 2 : (cg == 4 ? 4 : (cg == 2 ? 8 : 0));
    int best = 0;
    for (int bx = WX; bx < WX + 16; ++bx)
        for (int by = (WY + 2) & ~1; by < WY + 18; by += 2) {
            if (bx > g.nf[0] || by > g.nf[1] || bx > 256 || by > 256) continue;
            if ((bx * by) % mod != want) continue;
            if (best == 0 || bx * by < best) {
                best = bx * by;
                t.BX = bx;
                t.BY = by;
            }
        }
    if (best == 0) return false;
    t.CS = t.BX * t.BY;
    // Coil passes per item: as many groups of cg coils as let two buffers fit in the
    // budget (two blocks per SM), so the sample weights and the per-item work are shared
    // by more coils (12 coils in groups of 4: one item of 3 passes instead of 3 items).
    constexpr size_t kBudget = 112 * 1024;
    const int groups = (g.n_coil + cg - 1) / cg;
    const size_t pass_bytes = (size_t)t.CS * cg * sizeof(float2);
    t.passes = 1;
    while (t.passes < groups && cg * (t.passes + 1) <= 256 && 2 * (t.passes + 1) * pass_bytes <= kBudget)
        ++t.passes;
    const int coils = cg * t.passes;
    t.n_cg = (g.n_coil + coils - 1) / coils;
    t.n_items = n_sub * t.n_cg;
    t.box_bytes = (uint32_t)t.CS * coils * (uint32_t)sizeof(float2);
    t.buf_elems = (uint32_t)((t.CS * coils + 15) & ~15);
    // as many buffers (2..4) as fit in 96 KB (measured: a third 36 KB buffer costs more in
    // blocks per SM than it gains in prefetch depth on the 8-coil 512^2 radial workload)
    const size_t buf_bytes = (size_t)t.buf_elems * sizeof(float2);
    t.stages = 2;
    while (t.stages < kTmaMaxStages && (size_t)(t.stages + 1) * buf_bytes <= 96 * 1024) ++t.stages;
    return true;
}

size_t tma_interp_smem_bytes(const TmaWin &t) { return (size_t)t.stages * t.buf_elems * sizeof(float2); }

static int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

cudaError_t launch_interp2d_tma(const InterpArgs &a, const TmaWin &t, const CUtensorMap &map, int coil_group,
                                int threads, uint32_t *status, cudaStream_t s) {
    if (t.n_items == 0) return cudaSuccess;
    const size_t smem = tma_interp_smem_bytes(t);
    cudaError_t err = cudaSuccess;
    GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
        auto kern = t.passes > 1 ? k_interp2d_tma<WT, CG, true> : k_interp2d_tma<WT, CG, false>;
        err = set_smem(kern, smem);
        int per_sm = 0;
        if (err == cudaSuccess) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
        if (err == cudaSuccess) {
            const int64_t blocks = std::min<int64_t>(t.n_items, (int64_t)std::max(per_sm, 1) * sm_count());
            kern<<<(unsigned)blocks, threads, smem, s>>>(a, map, t, status);
            err = cudaGetLastError();
        }
    }));
    return err;
}

cudaError_t launch_interp_grad(const GradArgs &a, int64_t n_sub, int coil_group, int threads, cudaStream_t s) {
    if (n_sub == 0) return cudaSuccess;
    const size_t smem = grad_smem_bytes(a.g, coil_group);
    const dim3 grid((unsigned)n_sub, (unsigned)((a.g.n_coil + coil_group - 1) / coil_group));
    // dw/dx = w * (-2 beta d / h) with beta = beta2 / log2(e), h = 2 pi / nf
    float dsc[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < a.g.dim; ++d) {
        const double beta = (double)a.g.beta2[d] / 1.4426950408889634;
        const double h = 6.283185307179586 / a.g.nf[d];
        dsc[d] = (float)(-2.0 * beta / h);
    }
    cudaError_t err = cudaSuccess;
    if (use_2d_path(a.g)) {  // warp per sample, lanes = coils x tap slots
        GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
            auto kern = k_interp_grad2d<WT, CG>;
            err = set_smem(kern, smem);
            if (err == cudaSuccess) {
                kern<<<grid, threads, smem, s>>>(a, dsc[0], dsc[1]);
                err = cudaGetLastError();
            }
        }));
        return err;
    }
    GBN_DISPATCH_D(a.g.dim, GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
        auto kern = k_interp_grad<D, WT, CG>;
        err = set_smem(kern, smem);
        if (err == cudaSuccess) {
            kern<<<grid, threads > 256 ? 256 : threads, smem, s>>>(a, dsc[0], dsc[1], dsc[2]);
            err = cudaGetLastError();
        }
    })));
    return err;
}

}  // namespace gbn
