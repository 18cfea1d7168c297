// Solver kernels: the vector work of linear CG (CG-SENSE) and of mripy's IST/FISTA with a
// Haar-wavelet soft threshold, so that a whole solver iteration runs on the GPU with its
// scalars in device memory (one CUDA graph per iteration, no host synchronisation).
//
//  * CG: r = rhs - A x, p = r; per iteration alpha = <r,r>/Re<p,Ap>, x += alpha p,
//    r -= alpha Ap, beta = <r,r>_new/<r,r>, p = r + beta p.  Inner products are summed in
//    FP64: per-block partials, then the last block to finish adds them in block order
//    (deterministic for a given vector length) and writes the scalars.  The reference has
//    no CG-SENSE routine (its linear CG on the normal equations, pics/proximal_func.py:
//    379-406, is commented out); this is that algorithm with forward_backward as A.
//  * IST/FISTA step (pics/CS_MRI_solvers_func.py:75-86 IST_32, :207-224 FIST_32): the
//    gradient update acc -= step (A^H A x - A^H b), the prox x = invT(soft(T acc, th))
//    (pics/proximal_func.py:46-52, soft threshold :20-24: v / (|v| + 1e-6) * max(|v| - th, 0))
//    with T the orthonormal level-L Haar transform (DWTnd, pics/operators_class.py:394-416,
//    wavelet 'haar'), and FISTA's momentum y = x + (t_k - 1)/t_{k+1} (x - x_pre).  A level-L
//    Haar transform maps each tile of 2^L cells per axis onto itself, so one block takes
//    whole tiles: level 1 runs in registers on 2^DIM cubes read straight from the vectors
//    (its thresholded bands stay there), levels 2..L on the approximations in shared
//    memory, then the inverse back out: one read and one write of each vector per step.
//  * gbn_haar_dwt: the same tile transform, writing (or reading) the coefficients in the
//    layout of pywt.coeffs_to_array (approximation block first along every axis, then the
//    detail blocks of the coarsest level, ..., the finest level's last).
#include <cmath>
#include <string>

#include "common.cuh"

namespace gbn {
namespace {

constexpr int kVecThreads = 256;
constexpr int kHaarThreads = 256;
constexpr int kHaarMaxElems = 4096;     // complex elements per block (32 KB of shared memory)
constexpr int kHaarBlockElems = 2048;   // elements per block when tiles are smaller than that

int vec_blocks(int64_t n) {
    const int64_t b = (n + kVecThreads - 1) / kVecThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, kRedBlocks));
}

// block-wide FP64 sum; the result is valid in thread 0.  Fixed order for a given blockDim.
__device__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();  // sh may still be read by a previous call
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// Adds this block's share v into the grid total.  Returns true in thread 0 of the last block
// to finish, with *total set to the sum of the per-block partials taken in block order; the
// done counter is reset for the next reduction.  No thread waits for another block.
__device__ bool grid_sum(double v, double *partial, unsigned *done, double *total) {
    __shared__ double sh[32];
    __shared__ bool last;
    const double b = block_sum(v, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = b;
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += __ldcg(&partial[i]);
    s = block_sum(s, sh);
    if (threadIdx.x != 0) return false;
    *done = 0;
    *total = s;
    return true;
}

__global__ void __launch_bounds__(kVecThreads) k_cg_start(const float2 *__restrict__ rhs,
                                                          const float2 *__restrict__ q, float2 *__restrict__ r,
                                                          float2 *__restrict__ p, int64_t n, double *partial,
                                                          SolveState *st) {
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float2 v = rhs[i];
        if (q) {
            const float2 w = q[i];
            v.x -= w.x;
            v.y -= w.y;
        }
        r[i] = v;
        p[i] = v;
        acc += (double)v.x * v.x + (double)v.y * v.y;
    }
    double tot;
    if (grid_sum(acc, partial, &st->done, &tot)) {
        st->rs = tot;
        st->alpha = 0.0;
        st->beta = 0.0;
        st->t = 1.0;
        st->it = 0;
    }
}

__global__ void __launch_bounds__(kVecThreads) k_cg_alpha(const float2 *__restrict__ p, const float2 *__restrict__ q,
                                                          int64_t n, double *partial, SolveState *st) {
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 a = p[i], b = q[i];
        acc += (double)a.x * b.x + (double)a.y * b.y;  // Re(conj(p) q)
    }
    double pq;
    if (grid_sum(acc, partial, &st->done, &pq)) {
        const double a = st->rs / pq;
        // an exactly converged residual (rs = 0) or a vanishing curvature leaves x where it is
        st->alpha = (st->rs > 0.0 && pq != 0.0 && isfinite(a)) ? a : 0.0;
    }
}

__global__ void __launch_bounds__(kVecThreads) k_cg_update(float2 *__restrict__ x, float2 *__restrict__ r,
                                                           const float2 *__restrict__ p,
                                                           const float2 *__restrict__ q, int64_t n,
                                                           double *partial, SolveState *st, double *norms,
                                                           int cap) {
    const float a = (float)st->alpha;
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 pv = p[i], qv = q[i];
        float2 xv = x[i], rv = r[i];
        xv.x += a * pv.x;
        xv.y += a * pv.y;
        rv.x -= a * qv.x;
        rv.y -= a * qv.y;
        x[i] = xv;
        r[i] = rv;
        acc += (double)rv.x * rv.x + (double)rv.y * rv.y;
    }
    double rs_new;
    if (grid_sum(acc, partial, &st->done, &rs_new)) {
        const double b = rs_new / st->rs;
        st->beta = (st->rs > 0.0 && isfinite(b)) ? b : 0.0;
        st->rs = rs_new;
        if (norms && st->it < cap) norms[st->it] = sqrt(rs_new);
        st->it += 1;
    }
}

__global__ void __launch_bounds__(kVecThreads) k_cg_direction(const float2 *__restrict__ r, float2 *__restrict__ p,
                                                              int64_t n, const SolveState *st) {
    const float b = (float)st->beta;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 rv = r[i];
        float2 pv = p[i];
        pv.x = rv.x + b * pv.x;
        pv.y = rv.y + b * pv.y;
        p[i] = pv;
    }
}

// FIST_32's start (CS_MRI_solvers_func.py:207-211): y = step * rhs, y_acc = 0, x_pre = y, t = 1
__global__ void __launch_bounds__(kVecThreads) k_fista_start(const float2 *__restrict__ rhs, float step,
                                                             float2 *__restrict__ y, float2 *__restrict__ y_acc,
                                                             float2 *__restrict__ x_pre, int64_t n,
                                                             SolveState *st) {
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i0 == 0) {
        st->t = 1.0;
        st->done = 0;
        st->it = 0;
    }
    for (int64_t i = i0; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 b = rhs[i];
        const float2 v = make_float2(step * b.x, step * b.y);
        y[i] = v;
        x_pre[i] = v;
        y_acc[i] = make_float2(0.f, 0.f);
    }
}

__global__ void __launch_bounds__(kVecThreads) k_scale(const float2 *__restrict__ in, float a,
                                                       float2 *__restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = in[i];
        out[i] = make_float2(a * v.x, a * v.y);
    }
}

// ---- Pipe-Menon density compensation --------------------------------------------------
// w <- w / |C w| with C w = interp(spread(w)) on the plan's Gaussian kernel; w is held as
// complex samples (imaginary part 0) so the plan's spread reads it directly.
__global__ void __launch_bounds__(kVecThreads) k_dcf_fill(float2 *__restrict__ w, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        w[i] = make_float2(1.f, 0.f);
}

__global__ void __launch_bounds__(kVecThreads) k_dcf_update(float2 *__restrict__ w, const float2 *__restrict__ cw,
                                                            int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 c = cw[i];
        const float a = sqrtf(c.x * c.x + c.y * c.y);
        // every sample's own stencil contributes w_j * sum_m g^2 > 0, so a > 0 unless w underflowed
        w[i] = make_float2(a > 0.f ? w[i].x / a : 0.f, 0.f);
    }
}

// dcf = w * M_g / sum_g(w) (mean 1 over each trajectory group).  Grid (kDcfBlocks, n_traj):
// block b of group g sums chunk b of the group in FP64, then every block adds the group's
// kDcfBlocks partials in block order (deterministic) and scales its chunk.
constexpr int kDcfBlocks = kDcfPartials;

__device__ __forceinline__ void dcf_chunk(const int64_t *off, int64_t &lo, int64_t &hi) {
    const int64_t a = off[blockIdx.y], b = off[blockIdx.y + 1];
    const int64_t chunk = (b - a + kDcfBlocks - 1) / kDcfBlocks;
    lo = min(b, a + chunk * blockIdx.x);
    hi = min(b, lo + chunk);
}

__global__ void __launch_bounds__(kVecThreads) k_dcf_partial(const float2 *__restrict__ w, const int64_t *off,
                                                             double *partial) {
    __shared__ double sh[32];
    int64_t lo, hi;
    dcf_chunk(off, lo, hi);
    double s = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += (double)w[i].x;
    s = block_sum(s, sh);
    if (threadIdx.x == 0) partial[(int64_t)blockIdx.y * kDcfBlocks + blockIdx.x] = s;
}

__global__ void __launch_bounds__(kVecThreads) k_dcf_scale(const float2 *__restrict__ w, const int64_t *off,
                                                           const double *partial, float *__restrict__ dcf) {
    __shared__ float scale;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < kDcfBlocks; ++i) s += partial[(int64_t)blockIdx.y * kDcfBlocks + i];
        const double n = (double)(off[blockIdx.y + 1] - off[blockIdx.y]);
        scale = s > 0.0 ? (float)(n / s) : 0.f;
    }
    __syncthreads();
    int64_t lo, hi;
    dcf_chunk(off, lo, hi);
    const float f = scale;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) dcf[i] = w[i].x * f;
}

// ---- Haar tiles ------------------------------------------------------------------------
// A level-L Haar transform maps each tile of T = 2^L cells per axis onto itself.  Blocks
// take whole units, a unit being (image, tile, channel chunk) with the chunk fastest, so the
// chunks of one tile run side by side and share the cache lines of interleaved channels.
//
// Inside a block the transform runs in place on 2^DIM cubes: level l combines the cells
// base + h*bits (h = 2^(l-1), base a multiple of 2h along every axis) into the approximation,
// kept at base, and the 2^DIM - 1 detail bands at the other corners.  Level 1 runs in
// registers on cubes loaded straight from the image (the prox keeps its thresholded details
// there); levels 2..L run on the approximation lattice in shared memory, one barrier each.
// Shared memory holds a unit's cells as [cell][channel], cell = in-tile (x, y, z) with L bits
// per axis and the last axis fastest.
struct TileRef {
    int64_t base;  // element of (image, channel chunk start, pixel 0)
    int64_t tcp;   // tile coordinates, 21 bits per axis
    int nch;       // channels of the chunk that exist (<= cpb)
};
constexpr int kHaarMaxUnits = 512;

template <int DIM>
__device__ __forceinline__ TileRef haar_unit(const HaarGeom &h, int64_t u) {
    const int64_t chunk = u % h.chunks;
    int64_t r = u / h.chunks;
    const int64_t tile = r % h.tiles_img;
    const int64_t outer = r / h.tiles_img;
    int64_t tr = tile, packed = 0;
#pragma unroll
    for (int d = DIM - 1; d >= 0; --d) {
        packed |= (tr % h.nt[d]) << (21 * d);
        tr /= h.nt[d];
    }
    const int64_t c0 = chunk * h.cpb;
    const int64_t left = h.inner - c0;
    return TileRef{outer * h.P * h.inner + c0, packed, (int)(left < h.cpb ? left : h.cpb)};
}

__device__ __forceinline__ int tile_coord(int64_t packed, int d) { return (int)((packed >> (21 * d)) & 0x1FFFFF); }

// image element of in-tile cell (coordinates c[]) and channel ch of a unit
template <int DIM>
__device__ __forceinline__ int64_t haar_pix_addr(const HaarGeom &h, const TileRef &t, const int *c, int ch) {
    const int T = 1 << h.L;
    int64_t pix = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) pix = pix * h.s[d] + (int64_t)tile_coord(t.tcp, d) * T + c[d];
    return t.base + pix * h.inner + ch;
}

// element of in-tile cell c[] (in-place layout) in pywt.coeffs_to_array's layout: the cell
// belongs to level l = the lowest level at which one of its coordinates is an odd multiple
// of 2^(l-1) (all coordinates 0: the level-L approximation), band bit b_d = (c_d >> (l-1)) & 1,
// position within the band c_d >> l; band (b_0..) of level l starts at (s_d >> l) * b_d
template <int DIM>
__device__ __forceinline__ int64_t haar_coeff_addr(const HaarGeom &h, const TileRef &t, const int *c, int ch) {
    int l = h.L;
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        if (c[d]) l = min(l, __ffs(c[d]));
    int64_t pix = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const int b = (c[d] >> (l - 1)) & 1;
        const int g = (b ? (h.s[d] >> l) : 0) + tile_coord(t.tcp, d) * (1 << (h.L - l)) + (c[d] >> l);
        pix = pix * h.s[d] + g;
    }
    return t.base + pix * h.inner + ch;
}

// in-tile cell coordinates of element e of a unit's cells (last axis fastest, L bits each)
template <int DIM>
__device__ __forceinline__ void cell_coords(int cell, int L, int *c) {
#pragma unroll
    for (int d = DIM - 1; d >= 0; --d) {
        c[d] = cell & ((1 << L) - 1);
        cell >>= L;
    }
}

// 2^DIM-point Haar butterflies on v[q], q's bit (DIM-1-d) selecting the upper cell along
// axis d; forward and inverse are the same orthonormal map, applied axis by axis (0 first)
template <int DIM>
__device__ __forceinline__ void cube_butterfly(float2 *v) {
    const float r2 = 0.70710678118654752440f;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const int bit = 1 << (DIM - 1 - d);
#pragma unroll
        for (int q = 0; q < (1 << DIM); ++q) {
            if (q & bit) continue;
            const float2 e = v[q], o = v[q | bit];
            v[q] = make_float2((e.x + o.x) * r2, (e.y + o.y) * r2);
            v[q | bit] = make_float2((e.x - o.x) * r2, (e.y - o.y) * r2);
        }
    }
}

__device__ __forceinline__ float2 soft_thresh(float2 v, float th) {
    const float a = sqrtf(v.x * v.x + v.y * v.y);
    const float s = fmaxf(a - th, 0.f) / (a + 1e-6f);
    return make_float2(v.x * s, v.y * s);
}

// Work item w of level l >= 1 in a block: channel (fastest), cube, unit.  Its cube corner
// cells are corner[d] = 2h * cube_d + h * bit_d with h = 2^(l-1).
struct CubeItem {
    int unit, ch;
    int corner[3];
};
template <int DIM>
__device__ __forceinline__ CubeItem cube_item(int w, int L, int l, int cpb_log) {
    CubeItem it;
    it.ch = w & ((1 << cpb_log) - 1);
    int r = w >> cpb_log;
    const int cb = L - l;  // bits per axis of the level's cube index
    const int cubes_log = DIM * cb;
    it.unit = r >> cubes_log;
    int cube = r & ((1 << cubes_log) - 1);
#pragma unroll
    for (int d = DIM - 1; d >= 0; --d) {
        it.corner[d] = (cube & ((1 << cb) - 1)) << l;
        cube >>= cb;
    }
    for (int d = DIM; d < 3; ++d) it.corner[d] = 0;
    return it;
}

// shared-memory element of cell c[] (plus offset h * bits(q)) of a unit, channel ch
template <int DIM>
__device__ __forceinline__ int sm_index(const CubeItem &it, int q, int h, int L, int cpb_log) {
    int cell = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) cell = (cell << L) | (it.corner[d] + (((q >> (DIM - 1 - d)) & 1) ? h : 0));
    return (((it.unit << (DIM * L)) | cell) << cpb_log) | it.ch;
}

// levels 2..L (forward) or L..2 (inverse) on the approximation lattice in shared memory;
// with th >= 0 the forward pass soft-thresholds each level's details, and the level-L
// approximation, as they are produced
template <int DIM, bool INV>
__device__ void haar_levels_smem(float2 *sm, int L, int cpb_log, int n_units, float th) {
    for (int step = 0; step < L - 1; ++step) {
        const int l = INV ? L - step : 2 + step;
        const int h = 1 << (l - 1);
        const int items = n_units << (DIM * (L - l) + cpb_log);
        for (int w = threadIdx.x; w < items; w += kHaarThreads) {
            const CubeItem it = cube_item<DIM>(w, L, l, cpb_log);
            float2 v[1 << DIM];
            int idx[1 << DIM];
#pragma unroll
            for (int q = 0; q < (1 << DIM); ++q) {
                idx[q] = sm_index<DIM>(it, q, h, L, cpb_log);
                v[q] = sm[idx[q]];
            }
            cube_butterfly<DIM>(v);
            if (!INV && th >= 0.f) {
#pragma unroll
                for (int q = 0; q < (1 << DIM); ++q)
                    if (q || l == L) v[q] = soft_thresh(v[q], th);
            }
#pragma unroll
            for (int q = 0; q < (1 << DIM); ++q) sm[idx[q]] = v[q];
        }
        __syncthreads();
    }
}

constexpr int kHaarCubes = 16;  // level-1 cubes per thread, times 2^DIM (4096-cell blocks, 256 threads)
static_assert(kHaarCubes * kHaarThreads == kHaarMaxElems, "a block's level-1 cubes must fit its threads");

// first unit of the block, the number of units it holds, and their decoded references
template <int DIM>
__device__ __forceinline__ int haar_block_units(const HaarGeom &h, TileRef *units) {
    const int64_t u0 = (int64_t)blockIdx.x << h.upb_log;
    const int64_t left = h.n_units - u0;
    const int nu = left < ((int64_t)1 << h.upb_log) ? (int)left : (1 << h.upb_log);
    for (int t = threadIdx.x; t < nu; t += kHaarThreads) units[t] = haar_unit<DIM>(h, u0 + t);
    return nu;
}

// global elements of a level-1 cube's 2^DIM cells
template <int DIM>
__device__ __forceinline__ void cube_addrs(const HaarGeom &h, const TileRef &t, const CubeItem &it, int64_t *g) {
    int c[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) c[d] = it.corner[d];
    const int64_t g0 = haar_pix_addr<DIM>(h, t, c, it.ch);
    int64_t stride = h.inner;
    int64_t off[3];
#pragma unroll
    for (int d = DIM - 1; d >= 0; --d) {
        off[d] = stride;
        stride *= h.s[d];
    }
#pragma unroll
    for (int q = 0; q < (1 << DIM); ++q) {
        int64_t a = g0;
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            if ((q >> (DIM - 1 - d)) & 1) a += off[d];
        g[q] = a;
    }
}

template <int DIM, bool MOM>
__global__ void __launch_bounds__(kHaarThreads, 4) k_haar_step(HaarStepArgs a) {
    constexpr int NQ = 1 << DIM;
    constexpr int CPT = kHaarCubes >> DIM;
    extern __shared__ float2 sm[];
    const HaarGeom &h = a.h;
    const int L = h.L, cpb_log = __ffs(h.cpb) - 1;
    __shared__ TileRef units[kHaarMaxUnits];
    __shared__ float c_mom;
    __shared__ double t_next;
    if (MOM && threadIdx.x == 0) {
        // t_{k+1} = (1 + sqrt(1 + 4 t_k^2)) / 2 (CS_MRI_solvers_func.py:219), in FP64 as numpy
        const double t = a.st->t;
        t_next = (1.0 + sqrt(1.0 + 4.0 * t * t)) / 2.0;
        c_mom = (float)((t - 1.0) / t_next);
    }
    const int nu = haar_block_units<DIM>(h, units);
    __syncthreads();
    const float cm = MOM ? c_mom : 0.f;
    // one element: gradient update, then (after the transform) the output with momentum
    auto load = [&](int64_t g) {
        float2 v = a.acc[g];
        if (a.q) {
            const float2 qv = a.q[g], b = a.rhs[g];
            v.x -= a.step * (qv.x - b.x);
            v.y -= a.step * (qv.y - b.y);
            a.acc[g] = v;
        }
        return v;
    };
    auto store = [&](int64_t g, float2 x) {
        if (MOM) {
            const float2 xp = a.x_pre[g];
            a.y[g] = make_float2(x.x + cm * (x.x - xp.x), x.y + cm * (x.y - xp.y));
            a.x_pre[g] = x;
        } else {
            a.x_out[g] = x;
        }
    };
    if (L == 0) {
        // plain soft threshold, element by element
        const int n = nu << cpb_log;
        for (int e = threadIdx.x; e < n; e += kHaarThreads) {
            const TileRef &t = units[e >> cpb_log];
            const int ch = e & (h.cpb - 1);
            if (ch >= t.nch) continue;
            const int c[3] = {0, 0, 0};
            const int64_t g = haar_pix_addr<DIM>(h, t, c, ch);
            store(g, soft_thresh(load(g), a.th));
        }
    } else {
        const int items = nu << (DIM * (L - 1) + cpb_log);
        float2 det[CPT][NQ];  // level-1 bands, thresholded (the approximation too when L == 1)
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
            const int w = threadIdx.x + j * kHaarThreads;
            if (w >= items) continue;
            const CubeItem it = cube_item<DIM>(w, L, 1, cpb_log);
            const TileRef &t = units[it.unit];
            const bool ok = it.ch < t.nch;
            int64_t g[NQ];
            cube_addrs<DIM>(h, t, it, g);
            float2 v[NQ];
#pragma unroll
            for (int q = 0; q < NQ; ++q) v[q] = ok ? load(g[q]) : make_float2(0.f, 0.f);
            cube_butterfly<DIM>(v);
#pragma unroll
            for (int q = 1; q < NQ; ++q) det[j][q] = soft_thresh(v[q], a.th);
            if (L == 1)
                det[j][0] = soft_thresh(v[0], a.th);
            else
                sm[sm_index<DIM>(it, 0, 1, L, cpb_log)] = v[0];
        }
        __syncthreads();
        haar_levels_smem<DIM, false>(sm, L, cpb_log, nu, a.th);
        haar_levels_smem<DIM, true>(sm, L, cpb_log, nu, -1.f);
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
            const int w = threadIdx.x + j * kHaarThreads;
            if (w >= items) continue;
            const CubeItem it = cube_item<DIM>(w, L, 1, cpb_log);
            const TileRef &t = units[it.unit];
            if (it.ch >= t.nch) continue;
            float2 v[NQ];
            v[0] = L == 1 ? det[j][0] : sm[sm_index<DIM>(it, 0, 1, L, cpb_log)];
#pragma unroll
            for (int q = 1; q < NQ; ++q) v[q] = det[j][q];
            cube_butterfly<DIM>(v);
            int64_t g[NQ];
            cube_addrs<DIM>(h, t, it, g);
#pragma unroll
            for (int q = 0; q < NQ; ++q) store(g[q], v[q]);
        }
    }
    if (MOM) {
        // the last block to finish stores t_{k+1}; every block read t_k before its increment
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&a.st->done, 1u) == gridDim.x - 1) {
                a.st->t = t_next;
                a.st->done = 0;
            }
        }
    }
}

template <int DIM, bool INV>
__global__ void __launch_bounds__(kHaarThreads) k_haar_dwt(HaarGeom h, const float2 *__restrict__ in,
                                                           float2 *__restrict__ out) {
    constexpr int NQ = 1 << DIM;
    extern __shared__ float2 sm[];
    const int L = h.L, cpb_log = __ffs(h.cpb) - 1;
    __shared__ TileRef units[kHaarMaxUnits];
    const int nu = haar_block_units<DIM>(h, units);
    __syncthreads();
    const int cell_log = DIM * L;
    const int n_el = nu << (cell_log + cpb_log);
    if (L == 0) {
        for (int e = threadIdx.x; e < n_el; e += kHaarThreads) {
            const TileRef &t = units[e >> cpb_log];
            const int ch = e & (h.cpb - 1);
            if (ch >= t.nch) continue;
            const int c[3] = {0, 0, 0};
            const int64_t g = haar_pix_addr<DIM>(h, t, c, ch);
            out[g] = in[g];
        }
        return;
    }
    const int items = nu << (DIM * (L - 1) + cpb_log);
    if (!INV) {
        for (int w = threadIdx.x; w < items; w += kHaarThreads) {
            const CubeItem it = cube_item<DIM>(w, L, 1, cpb_log);
            const TileRef &t = units[it.unit];
            const bool ok = it.ch < t.nch;
            int64_t g[NQ];
            cube_addrs<DIM>(h, t, it, g);
            float2 v[NQ];
#pragma unroll
            for (int q = 0; q < NQ; ++q) v[q] = ok ? in[g[q]] : make_float2(0.f, 0.f);
            cube_butterfly<DIM>(v);
#pragma unroll
            for (int q = 0; q < NQ; ++q) sm[sm_index<DIM>(it, q, 1, L, cpb_log)] = v[q];
        }
        __syncthreads();
        haar_levels_smem<DIM, false>(sm, L, cpb_log, nu, -1.f);
        for (int e = threadIdx.x; e < n_el; e += kHaarThreads) {
            const TileRef &t = units[e >> (cell_log + cpb_log)];
            const int ch = e & (h.cpb - 1);
            if (ch >= t.nch) continue;
            int c[3];
            cell_coords<DIM>((e >> cpb_log) & ((1 << cell_log) - 1), L, c);
            out[haar_coeff_addr<DIM>(h, t, c, ch)] = sm[e];
        }
    } else {
        for (int e = threadIdx.x; e < n_el; e += kHaarThreads) {
            const TileRef &t = units[e >> (cell_log + cpb_log)];
            const int ch = e & (h.cpb - 1);
            float2 v = make_float2(0.f, 0.f);
            if (ch < t.nch) {
                int c[3];
                cell_coords<DIM>((e >> cpb_log) & ((1 << cell_log) - 1), L, c);
                v = in[haar_coeff_addr<DIM>(h, t, c, ch)];
            }
            sm[e] = v;
        }
        __syncthreads();
        haar_levels_smem<DIM, true>(sm, L, cpb_log, nu, -1.f);
        for (int w = threadIdx.x; w < items; w += kHaarThreads) {
            const CubeItem it = cube_item<DIM>(w, L, 1, cpb_log);
            const TileRef &t = units[it.unit];
            if (it.ch >= t.nch) continue;
            float2 v[NQ];
#pragma unroll
            for (int q = 0; q < NQ; ++q) v[q] = sm[sm_index<DIM>(it, q, 1, L, cpb_log)];
            cube_butterfly<DIM>(v);
            int64_t g[NQ];
            cube_addrs<DIM>(h, t, it, g);
#pragma unroll
            for (int q = 0; q < NQ; ++q) out[g[q]] = v[q];
        }
    }
}

int64_t haar_blocks(const HaarGeom &h) { return (h.n_units + ((int64_t)1 << h.upb_log) - 1) >> h.upb_log; }
size_t haar_smem(const HaarGeom &h) { return (sizeof(float2) * h.cpb) << (h.dim * h.L + h.upb_log); }

}  // namespace

int haar_geom(int dim, const int32_t *shape, int level, int64_t n_outer, int64_t n_inner, HaarGeom &h) {
    if (dim < 1 || dim > 3) return record_error(GBN_ERR_ARG, "Haar transform: dim must be 1, 2 or 3");
    if (!shape || level < 0 || n_outer < 1 || n_inner < 1)
        return record_error(GBN_ERR_ARG, "Haar transform: bad shape, level or image count");
    if (dim * level > 12)
        return record_error(GBN_ERR_CAPACITY, "Haar transform: tiles of 2^level cells per axis above 4096 cells");
    h = HaarGeom{};
    h.dim = dim;
    h.L = level;
    h.P = 1;
    h.tiles_img = 1;
    for (int d = 0; d < 3; ++d) {
        h.s[d] = d < dim ? shape[d] : 1;
        if (d < dim && (h.s[d] < 1 || (h.s[d] & ((1 << level) - 1))))
            return record_error(GBN_ERR_ARG, "Haar transform: every axis size must be a multiple of 2^level");
        h.nt[d] = d < dim ? h.s[d] >> level : 1;
        if (h.nt[d] >= (1 << 21)) return record_error(GBN_ERR_CAPACITY, "Haar transform: more than 2^21 tiles along an axis");
        h.P *= h.s[d];
        h.tiles_img *= h.nt[d];
    }
    h.inner = n_inner;
    h.n_outer = n_outer;
    // channels per unit: interleaved channels of one tile side by side, within 4096 elements
    const int64_t cells = (int64_t)1 << (dim * level);
    h.cpb = 1;
    while (h.cpb * 2 <= n_inner && cells * h.cpb * 2 <= kHaarMaxElems) h.cpb *= 2;
    h.chunks = (n_inner + h.cpb - 1) / h.cpb;
    h.n_units = n_outer * h.tiles_img * h.chunks;
    // units per block: up to 2048 elements (one unit when a unit is larger)
    int upb_log = 0;
    while (((cells * h.cpb) << (upb_log + 1)) <= kHaarBlockElems && (1 << (upb_log + 1)) <= kHaarMaxUnits) ++upb_log;
    h.upb_log = upb_log;
    // the kernels give each thread at most kHaarCubes / 2^dim level-1 cubes of a block
    if (((cells * h.cpb) << upb_log) > kHaarMaxElems)
        return record_error(GBN_ERR_INTERNAL, "Haar transform: block above its element budget");
    if (haar_blocks(h) > 0x7fffffff) return record_error(GBN_ERR_CAPACITY, "Haar transform: too many tiles");
    return GBN_OK;
}

cudaError_t launch_cg_start(const float2 *rhs, const float2 *q, float2 *r, float2 *p, int64_t n, double *partial,
                            SolveState *st, cudaStream_t s) {
    k_cg_start<<<vec_blocks(n), kVecThreads, 0, s>>>(rhs, q, r, p, n, partial, st);
    return cudaGetLastError();
}
cudaError_t launch_cg_alpha(const float2 *p, const float2 *q, int64_t n, double *partial, SolveState *st,
                            cudaStream_t s) {
    k_cg_alpha<<<vec_blocks(n), kVecThreads, 0, s>>>(p, q, n, partial, st);
    return cudaGetLastError();
}
cudaError_t launch_cg_update(float2 *x, float2 *r, const float2 *p, const float2 *q, int64_t n, double *partial,
                             SolveState *st, double *norms, int cap, cudaStream_t s) {
    k_cg_update<<<vec_blocks(n), kVecThreads, 0, s>>>(x, r, p, q, n, partial, st, norms, cap);
    return cudaGetLastError();
}
cudaError_t launch_cg_direction(const float2 *r, float2 *p, int64_t n, const SolveState *st, cudaStream_t s) {
    k_cg_direction<<<vec_blocks(n), kVecThreads, 0, s>>>(r, p, n, st);
    return cudaGetLastError();
}
cudaError_t launch_fista_start(const float2 *rhs, float step, float2 *y, float2 *y_acc, float2 *x_pre, int64_t n,
                               SolveState *st, cudaStream_t s) {
    k_fista_start<<<vec_blocks(n), kVecThreads, 0, s>>>(rhs, step, y, y_acc, x_pre, n, st);
    return cudaGetLastError();
}
cudaError_t launch_scale(const float2 *in, float a, float2 *out, int64_t n, cudaStream_t s) {
    k_scale<<<vec_blocks(n), kVecThreads, 0, s>>>(in, a, out, n);
    return cudaGetLastError();
}
cudaError_t launch_dcf_fill(float2 *w, int64_t n, cudaStream_t s) {
    k_dcf_fill<<<vec_blocks(n), kVecThreads, 0, s>>>(w, n);
    return cudaGetLastError();
}
cudaError_t launch_dcf_update(float2 *w, const float2 *cw, int64_t n, cudaStream_t s) {
    k_dcf_update<<<vec_blocks(n), kVecThreads, 0, s>>>(w, cw, n);
    return cudaGetLastError();
}
cudaError_t launch_dcf_finish(const float2 *w, const int64_t *d_traj_off, int n_traj, double *partial, float *dcf,
                              cudaStream_t s) {
    if (n_traj < 1) return cudaSuccess;
    if (n_traj > 65535) return cudaErrorInvalidConfiguration;
    const dim3 grid(kDcfBlocks, n_traj);
    k_dcf_partial<<<grid, kVecThreads, 0, s>>>(w, d_traj_off, partial);
    k_dcf_scale<<<grid, kVecThreads, 0, s>>>(w, d_traj_off, partial, dcf);
    return cudaGetLastError();
}

cudaError_t launch_haar_step(const HaarStepArgs &a, bool momentum, cudaStream_t s) {
    const int64_t nb = haar_blocks(a.h);
    if (nb == 0) return cudaSuccess;
    const size_t sm = haar_smem(a.h);
#define GBN_HAAR_STEP(D)                                                                    \
    do {                                                                                    \
        if (momentum)                                                                       \
            k_haar_step<D, true><<<(unsigned)nb, kHaarThreads, sm, s>>>(a);                 \
        else                                                                                \
            k_haar_step<D, false><<<(unsigned)nb, kHaarThreads, sm, s>>>(a);                \
    } while (0)
    if (a.h.dim == 1)
        GBN_HAAR_STEP(1);
    else if (a.h.dim == 2)
        GBN_HAAR_STEP(2);
    else
        GBN_HAAR_STEP(3);
#undef GBN_HAAR_STEP
    return cudaGetLastError();
}

cudaError_t launch_haar_dwt(const HaarGeom &h, const float2 *in, float2 *out, bool inverse, cudaStream_t s) {
    const int64_t nb = haar_blocks(h);
    if (nb == 0) return cudaSuccess;
    const size_t sm = haar_smem(h);
#define GBN_HAAR_DWT(D)                                                                     \
    do {                                                                                    \
        if (inverse)                                                                        \
            k_haar_dwt<D, true><<<(unsigned)nb, kHaarThreads, sm, s>>>(h, in, out);         \
        else                                                                                \
            k_haar_dwt<D, false><<<(unsigned)nb, kHaarThreads, sm, s>>>(h, in, out);        \
    } while (0)
    if (h.dim == 1)
        GBN_HAAR_DWT(1);
    else if (h.dim == 2)
        GBN_HAAR_DWT(2);
    else
        GBN_HAAR_DWT(3);
#undef GBN_HAAR_DWT
    return cudaGetLastError();
}

}  // namespace gbn

using namespace gbn;

// ---- C ABI: standalone wavelet and soft threshold ---------------------------------------
int gbn_haar_dwt(int32_t dim, const int32_t *shape, int32_t level, int64_t n_outer, int64_t n_inner,
                 const void *in, void *out, int32_t inverse, gbn_stream_t stream) {
    HaarGeom h;
    if (int st = haar_geom(dim, shape, level, n_outer, n_inner, h)) return st;
    if (!in || !out) return record_error(GBN_ERR_ARG, "Haar transform: null buffer");
    if (in == out && level > 0)
        return record_error(GBN_ERR_ARG, "Haar transform: input and output must be different buffers");
    cudaError_t e = launch_haar_dwt(h, (const float2 *)in, (float2 *)out, inverse != 0, (cudaStream_t)stream);
    if (e != cudaSuccess) return record_error(GBN_ERR_CUDA, (std::string("Haar transform: ") + cudaGetErrorString(e)).c_str());
    return GBN_OK;
}

int gbn_prox_haar(int32_t dim, const int32_t *shape, int32_t level, int64_t n_outer, int64_t n_inner,
                  const void *in, float th, void *out, gbn_stream_t stream) {
    HaarGeom h;
    if (int st = haar_geom(dim, shape, level, n_outer, n_inner, h)) return st;
    if (!in || !out) return record_error(GBN_ERR_ARG, "Haar prox: null buffer");
    if (!(th >= 0.f) || !std::isfinite(th)) return record_error(GBN_ERR_ARG, "Haar prox: threshold must be finite and >= 0");
    HaarStepArgs a{};
    a.h = h;
    a.acc = (float2 *)in;  // read only: no gradient update (q == null)
    a.th = th;
    a.x_out = (float2 *)out;
    cudaError_t e = launch_haar_step(a, false, (cudaStream_t)stream);
    if (e != cudaSuccess) return record_error(GBN_ERR_CUDA, (std::string("Haar prox: ") + cudaGetErrorString(e)).c_str());
    return GBN_OK;
}
