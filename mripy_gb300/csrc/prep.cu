// Sample preparation and bin sorting (the set_points stage).
//
// For every sample the FP64 coordinate reduction of the reference is applied once
// (xi = x*df mod 2pi, m = 1 + xi // h, fft/nufft_func.py:562-565), and the result is
// stored as the first tap cell (m - nspread) mod nf and the in-cell fraction in FP32.
// The spread and interp kernels only ever see these packed records.
#include "common.cuh"

namespace gbn {

namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;

// Python float semantics of a % b and a // b for b > 0 (CPython float_rem /
// float_floor_div), so that the nearest-cell choice matches the reference.
__device__ inline double py_mod(double a, double b) {
    double m = fmod(a, b);
    if (m != 0.0) {
        if ((b < 0) != (m < 0)) m += b;
    } else {
        m = copysign(0.0, b);
    }
    return m;
}
__device__ inline double py_floordiv(double a, double b) {
    double m = fmod(a, b);
    double div = (a - m) / b;
    if (m != 0.0 && ((b < 0) != (m < 0))) div -= 1.0;
    double fd;
    if (div != 0.0) {
        fd = floor(div);
        if (div - fd > 0.5) fd += 1.0;
    } else {
        fd = copysign(0.0, a / b);
    }
    return fd;
}

__device__ inline int group_of(const int64_t *off, int n_traj, int64_t j) {
    int lo = 0, hi = n_traj;  // off[lo] <= j < off[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (off[mid] <= j) lo = mid; else hi = mid;
    }
    return lo;
}

template <typename T>
__global__ void k_prep(const T *__restrict__ x, const T *__restrict__ y, const T *__restrict__ z,
                       int64_t M, const int64_t *__restrict__ traj_off, Geom gs, Geom gi, double df,
                       float4 *__restrict__ pts, uint32_t *__restrict__ home_key,
                       uint32_t *__restrict__ touch_count, uint32_t *__restrict__ home_count,
                       uint32_t *__restrict__ status) {
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= M) return;
    const int dim = gs.dim, ns = gs.ns;
    const T *src[3] = {x, y, z};
    float f[3] = {0.f, 0.f, 0.f};
    int c0[3] = {0, 0, 0};
    bool bad = false;
    // loops over all three axes with a guard (not up to dim): unrolled, so the per-axis
    // arrays and the Geom fields are indexed by constants and stay out of local memory
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= dim) continue;
        double xs = (double)src[d][j] * df;
        if (!isfinite(xs)) { bad = true; continue; }
        const int nf = gs.nf[d];
        const double h = kTwoPi / nf;
        double xi = py_mod(xs, kTwoPi);
        int64_t m = 1 + (int64_t)py_floordiv(xi, h);
        double fr = (xi - h * (double)(m - 1)) / h;
        f[d] = (float)fr;
        int64_t first = (m - ns) % nf;
        if (first < 0) first += nf;
        c0[d] = (int)first;
    }
    if (bad) {
        atomicOr(status, 1u);
        for (int d = 0; d < 3; ++d) { f[d] = 0.f; c0[d] = 0; }
    }
    pts[j] = make_float4(f[0], f[1], f[2], __uint_as_float(pack_cells(dim, c0[0], c0[1], c0[2])));

    const int g = group_of(traj_off, gs.n_traj, j);
    int t[3] = {0, 0, 0};
    uint32_t touch = 1;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= dim) continue;
        int cc = c0[d] + ns - 1;
        if (cc >= gi.nf[d]) cc -= gi.nf[d];
        t[d] = cc / gi.tile[d];
        touch *= (uint32_t)touched_tiles(c0[d], gs.W, gs.nf[d], gs.tile[d], gs.ntile[d]);
    }
    uint32_t key = (uint32_t)g * (uint32_t)gi.ntiles +
                   (uint32_t)((t[0] * gi.ntile[1] + t[1]) * gi.ntile[2] + t[2]);
    home_key[j] = key;
    atomicAdd(&home_count[key], 1u);
    touch_count[j] = touch;
}

__global__ void k_dup_keys(const float4 *__restrict__ pts, int64_t M, const int64_t *__restrict__ traj_off,
                           Geom gs, const uint64_t *__restrict__ touch_off, uint32_t *__restrict__ keys,
                           uint32_t *__restrict__ vals, uint32_t *__restrict__ tile_count) {
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= M) return;
    const int dim = gs.dim;
    int c0[3];
    unpack_cells(dim, __float_as_uint(pts[j].w), c0[0], c0[1], c0[2]);
    int n[3] = {1, 1, 1}, t0[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= dim) continue;
        n[d] = touched_tiles(c0[d], gs.W, gs.nf[d], gs.tile[d], gs.ntile[d]);
        t0[d] = c0[d] / gs.tile[d];
    }
    const uint32_t base = (uint32_t)group_of(traj_off, gs.n_traj, j) * (uint32_t)gs.ntiles;
    uint64_t pos = touch_off[j];
    for (int a = 0; a < n[0]; ++a) {
        int ta = (t0[0] + a) % gs.ntile[0];
        for (int b = 0; b < n[1]; ++b) {
            int tb = (t0[1] + b) % gs.ntile[1];
            for (int q = 0; q < n[2]; ++q) {
                int tq = (t0[2] + q) % gs.ntile[2];
                uint32_t key = base + (uint32_t)((ta * gs.ntile[1] + tb) * gs.ntile[2] + tq);
                keys[pos] = key;
                vals[pos] = (uint32_t)j;
                atomicAdd(&tile_count[key], 1u);
                ++pos;
            }
        }
    }
}

__global__ void k_gather_pts(const float4 *__restrict__ pts, const uint32_t *__restrict__ idx, int64_t n,
                             float4 *__restrict__ out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = pts[idx[i]];
}

// per tile: its number of work items; optionally counts the work items of dense tiles
// (n_dense) and the tiles split over several items (n_split)
__global__ void k_count_subs(const uint32_t *__restrict__ count, int64_t n, int max_sub, int every_tile,
                             uint32_t dense_min, uint32_t *__restrict__ n_sub, uint32_t *n_dense,
                             uint32_t *n_split) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    uint32_t c = count[t];
    uint32_t s = (c + (uint32_t)max_sub - 1) / (uint32_t)max_sub;
    if (every_tile && s == 0) s = 1;
    n_sub[t] = s;
    if (n_dense && dense_min > 0 && c >= dense_min) atomicAdd(n_dense, s);
    if (n_split && s > 1) atomicAdd(n_split, 1u);
}

// interleave: the s > 1 items of a split tile take every s-th entry (item k: entries k,
// k + s, k + 2s, ...; stride s in the flags above kStrideShift) instead of consecutive runs,
// so that each item holds a spatially even share of the tile's samples
__global__ void k_build_subs(const uint32_t *__restrict__ count, const uint32_t *__restrict__ tile_off,
                             const uint32_t *__restrict__ sub_off, int64_t n, int max_sub, int every_tile,
                             uint32_t dense_min, int interleave, uint32_t *__restrict__ split_list,
                             uint32_t *__restrict__ split_cursor, uint32_t *__restrict__ dense_list,
                             uint32_t *__restrict__ dense_cursor, int4 *__restrict__ subs) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    uint32_t c = count[t];
    uint32_t s = (c + (uint32_t)max_sub - 1) / (uint32_t)max_sub;
    if (every_tile && s == 0) s = 1;
    uint32_t o = sub_off[t];
    const bool dense = dense_min > 0 && c >= dense_min;
    if (s > 1 && split_list) split_list[atomicAdd(split_cursor, 1u)] = (uint32_t)t;  // order is irrelevant
    if (dense && s > 0 && dense_list) {
        const uint32_t d = atomicAdd(dense_cursor, s);
        for (uint32_t k = 0; k < s; ++k) dense_list[d + k] = o + k;
    }
    for (uint32_t k = 0; k < s; ++k) {
        int flags = (s > 1 ? kSplitFlag : 0) | (k == 0 ? kFirstFlag : 0) | (dense ? kDenseFlag : 0);
        if (interleave && s > 1) {
            const uint32_t len = (c - k + s - 1) / s;  // entries k, k + s, ... below c
            subs[o + k] = make_int4((int)t, (int)(tile_off[t] + k), (int)len, flags | (int)(s << kStrideShift));
        } else {
            uint32_t start = k * (uint32_t)max_sub;
            uint32_t len = c > start ? min((uint32_t)max_sub, c - start) : 0u;
            subs[o + k] = make_int4((int)t, (int)(tile_off[t] + start), (int)len, flags);
        }
    }
}

inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

cudaError_t launch_prep(int coord_dtype, const void *x, const void *y, const void *z, int64_t M,
                        const int64_t *d_traj_off, const Geom &gs, const Geom &gi, double df,
                        float4 *pts, uint32_t *home_key, uint32_t *touch_count, uint32_t *home_count,
                        cudaStream_t s) {
    // status word lives right after home_count's last tile entry (allocated by the caller)
    uint32_t *status = home_count + (size_t)gi.ntiles * gi.n_traj;
    if (M == 0) return cudaSuccess;
    const int th = 256;
    if (coord_dtype == GBN_COORD_F64)
        k_prep<double><<<blocks_for(M, th), th, 0, s>>>((const double *)x, (const double *)y, (const double *)z,
                                                      M, d_traj_off, gs, gi, df, pts, home_key, touch_count,
                                                      home_count, status);
    else
        k_prep<float><<<blocks_for(M, th), th, 0, s>>>((const float *)x, (const float *)y, (const float *)z,
                                                     M, d_traj_off, gs, gi, df, pts, home_key, touch_count,
                                                     home_count, status);
    return cudaGetLastError();
}

cudaError_t launch_dup_keys(const float4 *pts, int64_t M, const int64_t *d_traj_off, int n_traj,
                            const Geom &gs, const uint64_t *touch_off, uint32_t *keys, uint32_t *vals,
                            uint32_t *tile_count, cudaStream_t s) {
    (void)n_traj;
    if (M == 0) return cudaSuccess;
    k_dup_keys<<<blocks_for(M, 256), 256, 0, s>>>(pts, M, d_traj_off, gs, touch_off, keys, vals, tile_count);
    return cudaGetLastError();
}

cudaError_t launch_gather_pts(const float4 *pts, const uint32_t *idx, int64_t n, float4 *out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_gather_pts<<<blocks_for(n, 256), 256, 0, s>>>(pts, idx, n, out);
    return cudaGetLastError();
}

cudaError_t launch_count_subs(const uint32_t *count, int64_t n, int max_sub, int every_tile, uint32_t dense_min,
                              uint32_t *n_sub, uint32_t *n_dense, uint32_t *n_split, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_count_subs<<<blocks_for(n, 256), 256, 0, s>>>(count, n, max_sub, every_tile, dense_min, n_sub, n_dense,
                                                    n_split);
    return cudaGetLastError();
}

cudaError_t launch_build_subs(const uint32_t *count, const uint32_t *tile_off, const uint32_t *sub_off,
                              int64_t ntiles_total, int max_sub, int every_tile, uint32_t dense_min, int interleave,
                              uint32_t *split_list, uint32_t *split_cursor, uint32_t *dense_list,
                              uint32_t *dense_cursor, int4 *subs, cudaStream_t s) {
    if (ntiles_total == 0) return cudaSuccess;
    k_build_subs<<<blocks_for(ntiles_total, 256), 256, 0, s>>>(count, tile_off, sub_off, ntiles_total, max_sub,
                                                               every_tile, dense_min, interleave, split_list,
                                                               split_cursor, dense_list, dense_cursor, subs);
    return cudaGetLastError();
}

}  // namespace gbn
