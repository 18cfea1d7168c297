// Spread (type-1 gridding) launchers.
//
// 2-D / 3-D with at most 16 taps per dimension and 4 or 8 coils per block, on the tile shape
// they are built for: k_spread2d_reg / k_spread3d_reg (accumulators in registers).
// Other 2-D / 3-D tiles: k_spread2d / k_spread3d (warp-owned shared-memory rows, no atomics).
// Otherwise (1-D, wide stencils, small grids): k_spread (shared-memory atomics).
// 3-D with 8 coils per block also: k_spread_mma<3, ...> (tensor cores, 4 x 8 x 16 tiles) and
// k_spread3d_cube (register cubes), each followed by the compensated cube instance for the
// dense work items.
#include "dispatch.cuh"
#include "grid2d_kernels.cuh"
#include "grid3d_kernels.cuh"
#include "spread3d_cube.cuh"
#include "spread3d_mma.cuh"

#include <algorithm>

namespace gbn {

// the warp-row kernel uses signed tile-local coordinates, exact when nf >= tile + W
static bool use_2d_path(const Geom &g) {
    return g.dim == 2 && g.W <= 16 && g.nf[0] >= g.tile[0] + g.W && g.nf[1] >= g.tile[1] + g.W;
}

size_t spread_smem_bytes(const Geom &g, int coil_group) {
    if (use_2d_path(g)) return spread2d_smem_bytes(g, coil_group);
    if (grid3d_applies(g)) return spread3d_smem_bytes(g, coil_group);
    size_t cells = 1;
    for (int d = 0; d < g.dim; ++d) cells *= (size_t)g.tile[d];
    return cells * (size_t)coil_group * sizeof(float2);
}

cudaError_t launch_zero_split(const Geom &g, const uint32_t *split_tiles, int64_t n_split, float2 *grid,
                              cudaStream_t s) {
    if (n_split == 0 || g.n_coil == 0) return cudaSuccess;
    int cells = 1;
    for (int d = 0; d < g.dim; ++d) cells *= g.tile[d];
    const int th = cells >= 256 ? 256 : (cells >= 128 ? 128 : 64);
    const dim3 blocks((unsigned)n_split, (unsigned)(g.n_coil < 65535 ? g.n_coil : 65535));
    GBN_DISPATCH_D(g.dim, (k_zero_split<D><<<blocks, th, 0, s>>>(g, split_tiles, grid)));
    return cudaGetLastError();
}

// the 3-D register-tile kernel applies: (x, y) rows of 4 per warp, z run of 4 * 32/coils cells
static bool reg3d_path(const Geom &g, int coil_group, int threads) {
    return grid3d_applies(g) && (coil_group == 4 || coil_group == 8) && threads <= 256 && g.tile[1] % kRegRows == 0 &&
           g.tile[0] * g.tile[1] == kRegRows * (threads / 32) && g.tile[2] == kRegCols * (32 / coil_group);
}

// the cube kernel applies: 3-D, 8 coils per block, a tile of 8 or 16 cubes of 4^3 cells;
// returns its consumer warps (0 where it does not apply or was not chosen: the plan chooses
// it for its own default 3-D tile, a caller's tile takes it only with spread_variant 2)
static int cube_path(const Geom &g, int coil_group, int variant) {
    if (variant != 2 || !grid3d_applies(g) || coil_group != 8) return 0;
    for (int nwc : {8, 16})
        if (cube_tile_ok(g.tile, nwc)) return nwc;
    return 0;
}

// the tensor-core kernel applies: 8 coils per block, variant 3, its tile (3-D 4 x 8 x 16,
// 2-D 8 x 16) on a grid of at least tile + stencil cells per axis
static bool mma_path(const Geom &g, int coil_group, int variant) {
    if (variant != 3 || coil_group != 8) return false;
    if (g.dim == 3)
        return grid3d_applies(g) && g.tile[0] == kMmaTX && g.tile[1] == kMmaTY && g.tile[2] == kMmaTZ;
    return use_2d_path(g) && g.tile[0] == kMmaTY && g.tile[1] == kMmaTZ;
}

// the cube and tensor-core kernels read interleaved work items
bool spread_reads_interleaved(const Geom &g, int coil_group, int variant) {
    return cube_path(g, coil_group, variant) != 0 || mma_path(g, coil_group, variant);
}

int spread_path_kind(const Geom &g, int coil_group, int variant, int threads) {
    if (mma_path(g, coil_group, variant)) return 3;
    if (g.dim != 3 || coil_group != 8) return 0;
    if (cube_path(g, coil_group, variant)) return 2;
    return reg3d_path(g, coil_group, threads) ? 1 : 0;
}

int spread_kernel_count(const SpreadArgs &a, int64_t n_sub, int coil_group, int threads) {
    if (n_sub == 0) return 0;
    const bool two = cube_path(a.g, coil_group, a.variant) || mma_path(a.g, coil_group, a.variant) ||
                     reg3d_path(a.g, coil_group, threads);
    return (two && a.any_dense) ? 2 : 1;
}

// cube kernel instance: block b walks units b, b + gridDim.x, ...
template <int WT, int NWC, bool KAHAN>
static cudaError_t launch_cube_instance(const SpreadArgs &a, int64_t n_units, int n_cg, cudaStream_t s) {
    const CubeLayout L = cube_layout(a.g.tile, NWC);
    const int threads = (NWC + kCubeProducers) * 32;
    const int vec = ((uintptr_t)a.grid % 16 == 0) && (a.g.nf[2] % 2 == 0);
    auto kern = k_spread3d_cube<WT, NWC, KAHAN>;
    cudaError_t e = set_smem(kern, L.bytes);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, L.bytes);
    if (e != cudaSuccess) return e;
    // one unit per block: the hardware scheduler balances blocks of very unequal length.
    // (The kernel's loop also walks several units per block when launched with fewer
    // blocks; on the 2.56 M-sample 3-D radial workload, as many blocks as fit at once with
    // units assigned round robin measured 12.2 against 11.1 ms.)
    const int64_t blocks = n_units;
    (void)per_sm;
    kern<<<(unsigned)blocks, threads, L.bytes, s>>>(a, a.status, vec, n_units, n_cg);
    return cudaGetLastError();
}

template <int WT, int NWC>
static cudaError_t launch_cube(const SpreadArgs &a, int64_t n_sub, cudaStream_t s) {
    const int n_cg = (a.g.n_coil + 7) / 8;
    const int64_t n_units = n_sub * n_cg;
    cudaError_t e = launch_cube_instance<WT, NWC, false>(a, n_units, n_cg, s);
    if (e == cudaSuccess && a.any_dense) e = launch_cube_instance<WT, NWC, true>(a, n_units, n_cg, s);
    return e;
}

// tensor-core kernel: the plain instance (one block per unit), then the compensated one (one
// block per dense unit)
template <int WT, bool KAHAN>
static cudaError_t launch_mma_instance(const SpreadArgs &a, int64_t n_units, int n_cg, cudaStream_t s) {
    auto kern = k_spread_mma<3, WT, KAHAN>;
    const size_t smem = KAHAN ? kMmaSmemBytesK : kMmaSmemBytes;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    // the compensated instance: one block per (dense subproblem, coil group) only
    const int64_t blocks = KAHAN ? a.n_dense * n_cg : n_units;
    if (blocks == 0) return cudaSuccess;
    kern<<<(unsigned)blocks, mma_threads<KAHAN>(), smem, s>>>(a, a.status, n_cg);
    return cudaGetLastError();
}

template <int WT>
static cudaError_t launch_mma(const SpreadArgs &a, int64_t n_sub, cudaStream_t s) {
    const int n_cg = (a.g.n_coil + 7) / 8;
    const int64_t n_units = n_sub * n_cg;
    if (a.g.dim == 2) {  // no dense tiles in 2-D
        auto kern = k_spread_mma<2, WT, false>;
        cudaError_t e = set_smem(kern, kMmaSmemBytes);
        if (e != cudaSuccess) return e;
        kern<<<(unsigned)n_units, mma_threads<false>(), kMmaSmemBytes, s>>>(a, a.status, n_cg);
        return cudaGetLastError();
    }
    cudaError_t e = launch_mma_instance<WT, false>(a, n_units, n_cg, s);
    if (e == cudaSuccess && a.any_dense) e = launch_mma_instance<WT, true>(a, n_units, n_cg, s);
    return e;
}

cudaError_t launch_spread(const SpreadArgs &a, int64_t n_sub, int coil_group, int threads, cudaStream_t s) {
    if (n_sub == 0) return cudaSuccess;
    const size_t smem = spread_smem_bytes(a.g, coil_group);
    const dim3 grid((unsigned)n_sub, (unsigned)((a.g.n_coil + coil_group - 1) / coil_group));
    cudaError_t err = cudaSuccess;
    // tensor-core kernel (8 coils per block; 3-D: then compensated sums for dense units)
    if (mma_path(a.g, coil_group, a.variant)) {
        GBN_DISPATCH_W(a.g.W, { err = launch_mma<WT>(a, n_sub, s); });
        return err;
    }
    // register-tile kernel: 4 or 8 coils per block and the tile it is built for
    if (use_2d_path(a.g) && (coil_group == 4 || coil_group == 8) && threads <= 256 &&
        a.g.tile[0] == kRegRows * (threads / 32) &&
        a.g.tile[1] == kRegCols * (32 / coil_group)) {
        const size_t rsmem = spread2d_reg_smem_bytes(a.g, coil_group);
        GBN_DISPATCH_W(a.g.W, {
            if (coil_group == 8) {
                k_spread2d_reg<WT, 8><<<grid, threads, rsmem, s>>>(a);
            } else {
                k_spread2d_reg<WT, 4><<<grid, threads, rsmem, s>>>(a);
            }
            err = cudaGetLastError();
        });
        return err;
    }
    if (use_2d_path(a.g)) {
        GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
            auto kern = k_spread2d<WT, CG>;
            err = set_smem(kern, smem);
            if (err == cudaSuccess) {
                kern<<<grid, threads, smem, s>>>(a);
                err = cudaGetLastError();
            }
        }));
        return err;
    }
    // 3-D cube kernel (8 coils per block): plain sums, then (if any) compensated ones
    if (const int nwc = cube_path(a.g, coil_group, a.variant)) {
        GBN_DISPATCH_W(a.g.W, {
            err = nwc == 16 ? launch_cube<WT, 16>(a, n_sub, s) : launch_cube<WT, 8>(a, n_sub, s);
        });
        return err;
    }
    // 3-D register-tile kernel
    if (reg3d_path(a.g, coil_group, threads)) {
        // plain sums for ordinary tiles, then (if any) Kahan-compensated sums for dense ones
        const size_t rsmem = spread3d_reg_smem_bytes(a.g, coil_group);
        GBN_DISPATCH_W(a.g.W, {
            if (coil_group == 8) {
                k_spread3d_reg<WT, 8, false><<<grid, threads, rsmem, s>>>(a);
                if (a.any_dense) k_spread3d_reg<WT, 8, true><<<grid, threads, rsmem, s>>>(a);
            } else {
                k_spread3d_reg<WT, 4, false><<<grid, threads, rsmem, s>>>(a);
                if (a.any_dense) k_spread3d_reg<WT, 4, true><<<grid, threads, rsmem, s>>>(a);
            }
            err = cudaGetLastError();
        });
        return err;
    }
    if (grid3d_applies(a.g)) {
        GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
            auto kern = k_spread3d<WT, CG>;
            err = set_smem(kern, smem);
            if (err == cudaSuccess) {
                kern<<<grid, threads > 256 ? 256 : threads, smem, s>>>(a);
                err = cudaGetLastError();
            }
        }));
        return err;
    }
    GBN_DISPATCH_D(a.g.dim, GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
        auto kern = k_spread<D, WT, CG>;
        err = set_smem(kern, smem);
        if (err == cudaSuccess) {
            kern<<<grid, threads, smem, s>>>(a);
            err = cudaGetLastError();
        }
    })));
    return err;
}

}  // namespace gbn
