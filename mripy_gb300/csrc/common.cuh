// Internal definitions shared by the gbnufft CUDA translation units.
//
// Data layout in HBM (one plan):
//   grid      (n_traj * n_coil, nf1, nf2, nf3) complex64, instance-major, cuFFT-contiguous
//   pts       (M_total) float4 {f0, f1, f2, packed first-tap cells} per sample; f_d in [0, 1)
//             is the sample's position inside its grid cell, computed in FP64 from x*df mod 2pi
//   home list (M_total) samples sorted by (group, interp home bin): pts + sample index
//   dup list  (E) (sample, spread tile) pairs sorted by (group, tile): every tile a sample's
//             stencil touches, so each spread block owns a disjoint output tile
//   subs      int4 {tile id, start, length, flags} work items of <= max_subproblem samples
#pragma once

#include <cuda.h>  // CUtensorMap (TMA descriptors); the library calls no driver API directly
#include <cuda_runtime.h>
#include <stdint.h>

#include <nvtx3/nvToolsExt.h>  // header-only NVTX v3: stage ranges on a profiler's timeline

#include "../../include/gbnufft.h"

namespace gbn {

// NVTX range around one host-side stage (set_points, pad, FFT, interp, spread, crop): the
// stages show on a profiler's timeline; a few nanoseconds when no tool is attached
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

constexpr int kMaxW = 40;          // 2*nspread; nspread <= 20 (eps down to 1e-33 in 2-D gives 17)
constexpr int kSplitFlag = 1;      // tile is covered by more than one subproblem
constexpr int kFirstFlag = 2;      // first subproblem of its tile
constexpr int kDenseFlag = 4;      // tile above the dense-sample threshold: compensated sums
constexpr int kStrideShift = 8;    // flags >> kStrideShift: entry stride of an interleaved item (0: 1)
// default dense threshold (samples per 3-D spread tile).  Measured on GB300 for the 8-coil
// 20000 x 128 centre-out radial workload: 32768 flags 10% of the work items and costs 8% of
// the spread time; 2048 flags 41% and costs 27%.
constexpr int kDenseDefault = 32768;

struct Geom {
    int dim;
    int ns;          // nspread
    int W;           // taps per dim = 2*ns
    int nf[3];       // oversampled grid (1 beyond dim)
    int tile[3];     // tile size (cells) of the kernel this geometry serves
    int ntile[3];    // tiles per dim
    int ntiles;      // tiles per trajectory group
    float beta2[3];  // weight(d) = exp2(-beta2 * d^2), d in cells; beta = h^2/(4 tau), * log2(e)
    int64_t G;       // cells per instance
    int n_coil;
    int n_traj;
};

// ---- packed first-tap cell indices ------------------------------------------------------
// dim 1: c0 < 2^31; dim 2: c0, c1 < 2^16; dim 3: c0, c1 < 2^11, c2 < 2^10
__host__ __device__ inline uint32_t pack_cells(int dim, int c0, int c1, int c2) {
    if (dim == 1) return (uint32_t)c0;
    if (dim == 2) return (uint32_t)c0 | ((uint32_t)c1 << 16);
    return (uint32_t)c0 | ((uint32_t)c1 << 11) | ((uint32_t)c2 << 22);
}
__host__ __device__ inline void unpack_cells(int dim, uint32_t p, int &c0, int &c1, int &c2) {
    if (dim == 1) { c0 = (int)p; c1 = 0; c2 = 0; return; }
    if (dim == 2) { c0 = (int)(p & 0xFFFFu); c1 = (int)(p >> 16); c2 = 0; return; }
    c0 = (int)(p & 0x7FFu); c1 = (int)((p >> 11) & 0x7FFu); c2 = (int)(p >> 22);
}
inline bool cells_fit(int dim, const int nf[3]) {
    if (dim == 1) return nf[0] < (1 << 30);
    if (dim == 2) return nf[0] <= 65536 && nf[1] <= 65536;
    return nf[0] <= 2048 && nf[1] <= 2048 && nf[2] <= 1024;
}

// tiles a stencil of W cells starting at cell0 touches, walking forward with wrap
__host__ __device__ inline int touched_tiles(int cell0, int W, int nf, int T, int ntile) {
    int t = cell0 / T, pos = cell0, remaining = W, count = 0;
    while (remaining > 0 && count < ntile) {
        int tile_end = min((t + 1) * T, nf);
        int take = min(remaining, tile_end - pos);
        remaining -= take;
        ++count;
        pos = tile_end;
        ++t;
        if (pos >= nf) { pos = 0; t = 0; }
    }
    return count;
}

__device__ __forceinline__ int wrap_pos(int v, int n) {  // v in (-n, 2n)
    v = v < 0 ? v + n : v;
    return v >= n ? v - n : v;
}

// ---- internal launchers (defined in the .cu files) -------------------------------------
struct SortBuffers;

// api.cu: sets the calling thread's gbn_last_error message and returns code
int record_error(int code, const char *msg);

// prep.cu
cudaError_t launch_prep(int coord_dtype, const void *x, const void *y, const void *z, int64_t M,
                        const int64_t *d_traj_off, const Geom &gs, const Geom &gi, double df,
                        float4 *pts, uint32_t *home_key, uint32_t *touch_count, uint32_t *home_count,
                        cudaStream_t s);
cudaError_t launch_dup_keys(const float4 *pts, int64_t M, const int64_t *d_traj_off, int n_traj,
                            const Geom &gs, const uint64_t *touch_off, uint32_t *keys, uint32_t *vals,
                            uint32_t *tile_count, cudaStream_t s);
cudaError_t launch_gather_pts(const float4 *pts, const uint32_t *idx, int64_t n, float4 *out,
                              cudaStream_t s);
// dense_min > 0: subproblems of tiles with at least dense_min samples get kDenseFlag.
// split_list (may be null): the indices of the tiles covered by more than one subproblem
// are appended at *split_cursor (zeroed by the caller).
// interleave: split tiles' items take every s-th entry (only for the 3-D cube spread)
// dense_list (may be null): the indices of the items with kDenseFlag are appended at
// *dense_cursor (zeroed by the caller), in no particular order.
cudaError_t launch_build_subs(const uint32_t *count, const uint32_t *tile_off, const uint32_t *sub_off,
                              int64_t ntiles_total, int max_sub, int every_tile, uint32_t dense_min, int interleave,
                              uint32_t *split_list, uint32_t *split_cursor, uint32_t *dense_list,
                              uint32_t *dense_cursor, int4 *subs, cudaStream_t s);
// work items per tile; n_dense (may be null) accumulates the items of tiles with at least
// dense_min samples, n_split (may be null) the tiles split over several items
cudaError_t launch_count_subs(const uint32_t *count, int64_t n, int max_sub, int every_tile, uint32_t dense_min,
                              uint32_t *n_sub, uint32_t *n_dense, uint32_t *n_split, cudaStream_t s);

// grid.cu
struct SpreadArgs {
    Geom g;
    const int4 *subs;
    const float4 *pts;        // dup-list order
    const uint32_t *idx;      // dup-list sample index
    const float4 *pts_by_sample;  // the same records in the caller's sample order (41 MB for
                                  // 2.56 M samples: stays in L2), read through idx
    const float2 *c;          // samples
    int64_t c_elem, c_coil;   // strides (complex elements)
    const float *weight;      // per sample (original index) or null: density compensation
    float2 *grid;
    int any_dense;            // some subproblems carry kDenseFlag (compensated accumulation)
    const uint32_t *dense_subs;  // the indices of those subproblems (n_dense of them)
    int64_t n_dense;
    int variant;              // 3-D, 8 coils: 0 library choice, 1 warp rows, 2 cubes (gbn_plan_desc)
    uint32_t *status;         // the plan's status word (bounded waits of the cube kernel)
};
struct InterpArgs {
    Geom g;
    const int4 *subs;
    const float4 *pts;        // home order
    const uint32_t *idx;      // home order sample index
    const float2 *grid;
    float2 *c;
    int64_t c_elem, c_coil;
    const float *weight;      // per sample (original index) or null
};
struct GradArgs {
    Geom g;
    const int4 *subs;
    const float4 *pts;
    const uint32_t *idx;
    const float2 *grid;
    const float2 *gc;         // upstream gradient of the samples
    int64_t c_elem, c_coil;
    float *out;               // (M, dim)
    float scale;              // df
};
// the 3-D tensor-core interp: the spread's tiles and (sample, tile) work lists
struct MmaInterpArgs {
    Geom g;                       // the spread's geometry (4 x 8 x 16 tiles)
    const int4 *subs;             // the spread's work items
    const uint32_t *idx;          // (sample, tile) list: sample index per entry
    const float4 *pts_by_sample;  // per sample: in-cell fractions, first-tap cells
    const float2 *grid;
    float2 *c;                    // output samples (zeroed by the launcher)
    int64_t c_elem, c_coil;
    const float *weight;          // per sample or null
    int64_t M;                    // samples (all groups)
};
// whether the tensor-core interp takes this spread geometry and coil group
bool interp_mma_applies(const Geom &gs, int coil_group);
cudaError_t launch_interp3d_mma(const MmaInterpArgs &a, int64_t n_sub, uint32_t *status, cudaStream_t s);
cudaError_t launch_zero_split(const Geom &g, const uint32_t *split_tiles, int64_t n_split, float2 *grid,
                              cudaStream_t s);
cudaError_t launch_spread(const SpreadArgs &a, int64_t n_sub, int coil_group, int threads,
                          cudaStream_t s);
// the cube or tensor-core spread runs these arguments (the kernels that read interleaved
// work items)
bool spread_reads_interleaved(const Geom &g, int coil_group, int variant);
// the 3-D 8-coil spread kernel launch_spread runs: 3 tensor cores, 2 cubes, 1 warp rows, 0 other
int spread_path_kind(const Geom &g, int coil_group, int variant, int threads);
// kernels launch_spread runs for these arguments (the 3-D register path adds a Kahan instance)
int spread_kernel_count(const SpreadArgs &a, int64_t n_sub, int coil_group, int threads);
cudaError_t launch_interp(const InterpArgs &a, int64_t n_sub, int coil_group, int threads,
                          cudaStream_t s);
cudaError_t launch_interp_grad(const GradArgs &a, int64_t n_sub, int coil_group, int threads,
                               cudaStream_t s);
size_t spread_smem_bytes(const Geom &g, int coil_group);
size_t interp_smem_bytes(const Geom &g, int coil_group, int threads);
// shared memory of the plane-streaming 3-D interp, 0 where it does not apply
size_t interp3d_planes_smem(const Geom &g, int coil_group, int threads);
constexpr int kPlaneSamples = 64;  // samples per chunk of the plane-streaming 3-D interp
// plane box (y rows, z cells per coil) of the plane-streaming 3-D interp: the tensor copy's
// box over a grid tensor map (z, y, x, instance); false where the kernel does not apply
bool interp3d_plane_box(const Geom &g, int coil_group, int &BY, int &BZ);
// the plane-streaming 3-D interp; map (with status) may be null: the threads copy every plane
cudaError_t launch_interp3d_planes(const InterpArgs &a, int64_t n_sub, int coil_group, int threads,
                                   const CUtensorMap *map, uint32_t *status, cudaStream_t s);

// TMA-staged 2-D interp (interp2d_tma.cuh): window box geometry and launcher
struct TmaWin {
    int BX, BY;           // box: x rows, y cells per row (BY even, both cover the window)
    int CS;               // cells per coil in a staged window = BX * BY
    int n_cg;             // coil groups
    int64_t n_items;      // interp subproblems x coil groups
    uint32_t box_bytes;   // bytes one box copy delivers: BX * BY * CG * 8
    uint32_t buf_elems;   // float2 per buffer: CG * CS rounded up to 16 (128-byte buffers)
    int stages;           // window buffers per block (2..4)
    int passes;           // coil groups of CG per item: a window holds CG * passes coils
};
bool tma_window(const Geom &g, int coil_group, int64_t n_sub, TmaWin &t);
size_t tma_interp_smem_bytes(const TmaWin &t);
cudaError_t launch_interp2d_tma(const InterpArgs &a, const TmaWin &t, const CUtensorMap &map, int coil_group,
                                int threads, uint32_t *status, cudaStream_t s);

// deapod.cu
struct DeapodArgs {
    Geom g;                    // nf, dim, n_coil, n_traj
    int m[3];                  // image size (1 beyond dim)
    const float *tab[3];       // per-dim factor sqrt(pi/tau) exp(tau k^2) / nf_d, index i = k + m/2
    const float *grp_scale;    // per trajectory group (crop: 1/M_g) or null (= 1)
};
cudaError_t launch_build_tables(int dim, const int m[3], const int nf[3], double tau, float *tab0,
                                float *tab1, float *tab2, cudaStream_t s);
cudaError_t launch_pad(const DeapodArgs &a, const float2 *img, gbn_layout L, float2 *grid,
                       cudaStream_t s);
cudaError_t launch_crop(const DeapodArgs &a, const float2 *grid, float2 *img, gbn_layout L,
                        cudaStream_t s);
cudaError_t launch_pad_sense(const DeapodArgs &a, const float2 *x, gbn_layout XL, const float2 *sens,
                             gbn_layout SL, float2 *grid, cudaStream_t s);
cudaError_t launch_crop_sense(const DeapodArgs &a, const float2 *grid, const float2 *sens,
                              gbn_layout SL, float2 *x, gbn_layout XL, cudaStream_t s);

// solver.cu: vector kernels of the CG and IST/FISTA solvers
// Scalars of one solve, kept in device memory so no iteration waits on the host.
struct SolveState {
    double rs;       // <r, r> (CG)
    double alpha;    // rs / Re<p, Ap>
    double beta;     // rs_new / rs
    double t;        // FISTA t_k
    unsigned done;   // blocks of the running reduction that have finished (last-block test)
    int it;          // CG iterations completed = residual norms written
};
constexpr int kRedBlocks = 1216;  // upper bound on the blocks of one reduction (8 per SM)
cudaError_t launch_cg_start(const float2 *rhs, const float2 *q, float2 *r, float2 *p, int64_t n,
                            double *partial, SolveState *st, cudaStream_t s);
cudaError_t launch_cg_alpha(const float2 *p, const float2 *q, int64_t n, double *partial, SolveState *st,
                            cudaStream_t s);
cudaError_t launch_cg_update(float2 *x, float2 *r, const float2 *p, const float2 *q, int64_t n,
                             double *partial, SolveState *st, double *norms, int cap, cudaStream_t s);
cudaError_t launch_cg_direction(const float2 *r, float2 *p, int64_t n, const SolveState *st,
                                cudaStream_t s);
cudaError_t launch_fista_start(const float2 *rhs, float step, float2 *y, float2 *y_acc, float2 *x_pre,
                               int64_t n, SolveState *st, cudaStream_t s);
cudaError_t launch_scale(const float2 *in, float a, float2 *out, int64_t n, cudaStream_t s);
// Pipe-Menon density compensation: w = 1; w /= |interp(spread(w))|; dcf = w scaled to
// mean 1 per trajectory group
cudaError_t launch_dcf_fill(float2 *w, int64_t n, cudaStream_t s);
cudaError_t launch_dcf_update(float2 *w, const float2 *cw, int64_t n, cudaStream_t s);
constexpr int kDcfPartials = 64;  // FP64 partial sums per trajectory group (launch_dcf_finish)
cudaError_t launch_dcf_finish(const float2 *w, const int64_t *d_traj_off, int n_traj, double *partial, float *dcf,
                              cudaStream_t s);

// Images as Haar tiles: (n_outer, s0[, s1[, s2]], n_inner) complex64, contiguous; a
// level-L orthonormal Haar transform over the dim spatial axes acts on disjoint tiles of
// 2^L cells per axis, so one thread block holds whole tiles in shared memory.
struct HaarGeom {
    int dim;             // 1, 2 or 3 spatial axes
    int L;               // levels; tile edge T = 2^L
    int s[3];            // spatial sizes (1 beyond dim), s[dim-1] fastest
    int nt[3];           // tiles per axis = s >> L
    int64_t tiles_img;   // tiles per image
    int64_t n_outer;     // images (each with `inner` interleaved channels)
    int64_t inner;       // channels interleaved element by element (trailing axis)
    int64_t P;           // pixels per image
    int cpb;             // channels per unit (a power of two)
    int64_t chunks;      // channel chunks per image = ceil(inner / cpb)
    int64_t n_units;     // units = (image, tile, chunk), chunk fastest
    int upb_log;         // log2 units per thread block
};
int haar_geom(int dim, const int32_t *shape, int level, int64_t n_outer, int64_t n_inner, HaarGeom &h);
// one IST/FISTA step on Haar tiles (pics/CS_MRI_solvers_func.py:75-86, 207-224):
//   update:    acc -= step * (q - rhs)            (skipped when q is null)
//   prox:      x = H^-1 soft(H acc, th)           (proximal_func.py:20-24, 46-52)
//   momentum:  y = x + c (x - x_pre), x_pre = x   (FISTA; st->t advanced on the device)
//   else:      x_out = x
struct HaarStepArgs {
    HaarGeom h;
    float2 *acc;
    const float2 *q, *rhs;
    float step, th;
    float2 *x_out;             // IST
    float2 *x_pre, *y;         // FISTA
    SolveState *st;            // FISTA
};
cudaError_t launch_haar_step(const HaarStepArgs &a, bool momentum, cudaStream_t s);
cudaError_t launch_haar_dwt(const HaarGeom &h, const float2 *in, float2 *out, bool inverse, cudaStream_t s);

}  // namespace gbn
