// Gridding kernels: spread (type-1), interp (type-2) and the trajectory gradient.
//
// Weights.  Tap k (0 <= k < W = 2*nspread) of a sample with in-cell fraction f sits at
// distance d_k = f + (nspread - 1 - k) cells from the sample, and carries
// g = exp(-(h d_k)^2 / (4 tau)) = exp2(-beta2 * d_k^2), beta2 = h^2 log2(e) / (4 tau)
// (the reference's g(x) = exp(-x^2 / (4 tau)), fft/nufft_func.py:569-582).  The
// weights are separable, so each sample evaluates W exponentials per dimension in
// registers instead of the reference's FGG recurrences (E1 * E2^k * E3), which lose
// accuracy in FP32.
//
// Spread is output-stationary: a block owns one disjoint tile of the oversampled grid
// and accumulates the taps of every sample whose stencil reaches the tile (the dup
// list) in shared memory, then writes the tile once with coalesced stores.  Bins that
// are split over several blocks (dense k-space centre) flush with global atomics into
// a tile zeroed beforehand.  No global atomics otherwise, no separate grid memset.
//
// Interp stages the home bin's window (tile + W - 1 cells per dim, with periodic
// wrap) in shared memory for a group of coils, then each thread gathers one sample.
#pragma once

#include "common.cuh"

namespace gbn {

template <int D>
__device__ __forceinline__ void tile_coords(const Geom &g, int tile, int o[3], int e[3]) {
    int t2 = tile % g.ntile[2];
    int t1 = (tile / g.ntile[2]) % g.ntile[1];
    int t0 = tile / (g.ntile[2] * g.ntile[1]);
    int t[3] = {t0, t1, t2};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        o[d] = t[d] * g.tile[d];
        e[d] = d < D ? min(g.tile[d], g.nf[d] - o[d]) : 1;
    }
}

// weights of the W taps of one dimension
template <int WT>
__device__ __forceinline__ void tap_weights(float f, int ns, int W, float beta2, float *w) {
    const float base = f + (float)(ns - 1);
#pragma unroll
    for (int k = 0; k < (WT ? WT : kMaxW); ++k) {
        if (WT == 0 && k >= W) break;
        const float d = base - (float)k;
        w[k] = exp2f(-beta2 * d * d);
    }
}

// ------------------------------------------------------------------------- spread
template <int D, int WT, int CG>
__global__ void __launch_bounds__(512) k_spread(SpreadArgs a) {
    extern __shared__ float2 acc[];  // [tile cells][CG]
    const Geom &g = a.g;
    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    int o[3], e[3];
    tile_coords<D>(g, sub.x % g.ntiles, o, e);
    const int T1 = D > 1 ? g.tile[1] : 1, T2 = D > 2 ? g.tile[2] : 1;
    const int ncell = g.tile[0] * T1 * T2;
    for (int i = threadIdx.x; i < ncell * CG; i += blockDim.x) acc[i] = make_float2(0.f, 0.f);
    __syncthreads();

    const int W = WT ? WT : g.W;
    constexpr int WA = WT ? WT : kMaxW;
    for (int i = threadIdx.x; i < sub.z; i += blockDim.x) {
        const int64_t li = (int64_t)sub.y + i;
        const float4 p = a.pts[li];
        const uint32_t j = a.idx[li];
        int c0[3];
        unpack_cells(D, __float_as_uint(p.w), c0[0], c0[1], c0[2]);
        const float f[3] = {p.x, p.y, p.z};
        float w[D][WA];
        int r[3];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            tap_weights<WT>(f[d], g.ns, W, g.beta2[d], w[d]);
            int rr = c0[d] - o[d];
            r[d] = rr < 0 ? rr + g.nf[d] : rr;
        }
        float2 v[CG];
        const float sw = a.weight ? a.weight[j] : 1.f;
#pragma unroll
        for (int c = 0; c < CG; ++c) {
            const int coil = cg0 + c;
            v[c] = coil < g.n_coil ? a.c[(int64_t)j * a.c_elem + (int64_t)coil * a.c_coil] : make_float2(0.f, 0.f);
            v[c].x *= sw;
            v[c].y *= sw;
        }
        for (int k0 = 0; k0 < W; ++k0) {
            int l0 = r[0] + k0;
            if (l0 >= g.nf[0]) l0 -= g.nf[0];
            if (l0 >= e[0]) continue;
            const float w0 = w[0][k0];
            if constexpr (D == 1) {
                float2 *dst = acc + (size_t)l0 * CG;
#pragma unroll
                for (int c = 0; c < CG; ++c) {
                    atomicAdd(&dst[c].x, w0 * v[c].x);
                    atomicAdd(&dst[c].y, w0 * v[c].y);
                }
            } else {
                for (int k1 = 0; k1 < W; ++k1) {
                    int l1 = r[1] + k1;
                    if (l1 >= g.nf[1]) l1 -= g.nf[1];
                    if (l1 >= e[1]) continue;
                    const float w01 = w0 * w[1][k1];
                    if constexpr (D == 2) {
                        float2 *dst = acc + ((size_t)l0 * T1 + l1) * CG;
#pragma unroll
                        for (int c = 0; c < CG; ++c) {
                            atomicAdd(&dst[c].x, w01 * v[c].x);
                            atomicAdd(&dst[c].y, w01 * v[c].y);
                        }
                    } else {
#pragma unroll
                        for (int k2 = 0; k2 < WA; ++k2) {
                            if (WT == 0 && k2 >= W) break;
                            int l2 = r[2] + k2;
                            if (l2 >= g.nf[2]) l2 -= g.nf[2];
                            if (l2 >= e[2]) continue;
                            const float ww = w01 * w[2][k2];
                            float2 *dst = acc + (((size_t)l0 * T1 + l1) * T2 + l2) * CG;
#pragma unroll
                            for (int c = 0; c < CG; ++c) {
                                atomicAdd(&dst[c].x, ww * v[c].x);
                                atomicAdd(&dst[c].y, ww * v[c].y);
                            }
                        }
                    }
                }
            }
        }
    }
    __syncthreads();

    // flush the tile (only its in-grid extent) for each coil of the group
    const bool split = (sub.w & kSplitFlag) != 0;
    const int ecell = e[0] * e[1] * e[2];
    for (int c = 0; c < CG; ++c) {
        const int coil = cg0 + c;
        if (coil >= g.n_coil) break;
        float2 *dst = a.grid + ((int64_t)grp * g.n_coil + coil) * g.G;
        for (int i = threadIdx.x; i < ecell; i += blockDim.x) {
            const int l2 = i % e[2], l1 = (i / e[2]) % e[1], l0 = i / (e[2] * e[1]);
            const float2 val = acc[(((size_t)l0 * T1 + l1) * T2 + l2) * CG + c];
            const int64_t gi = ((int64_t)(o[0] + l0) * g.nf[1] + (o[1] + l1)) * g.nf[2] + (o[2] + l2);
            if (split) {
                atomicAdd(&dst[gi].x, val.x);
                atomicAdd(&dst[gi].y, val.y);
            } else {
                dst[gi] = val;
            }
        }
    }
}

// zero the tiles that several subproblems accumulate into: one block per (listed tile,
// coil); the list holds only split tiles (built when the points are set)
template <int D>
__global__ void k_zero_split(Geom g, const uint32_t *__restrict__ split_tiles, float2 *__restrict__ grid) {
    const uint32_t t = split_tiles[blockIdx.x];
    const int grp = (int)(t / (uint32_t)g.ntiles);
    int o[3], e[3];
    tile_coords<D>(g, (int)(t % (uint32_t)g.ntiles), o, e);
    const int ecell = e[0] * e[1] * e[2];
    for (int coil = blockIdx.y; coil < g.n_coil; coil += gridDim.y) {
        float2 *dst = grid + ((int64_t)grp * g.n_coil + coil) * g.G;
        for (int i = threadIdx.x; i < ecell; i += blockDim.x) {
            const int l2 = i % e[2], l1 = (i / e[2]) % e[1], l0 = i / (e[2] * e[1]);
            dst[((int64_t)(o[0] + l0) * g.nf[1] + (o[1] + l1)) * g.nf[2] + (o[2] + l2)] = make_float2(0.f, 0.f);
        }
    }
}

// ------------------------------------------------------------------------- interp window
template <int D, int CG>
__device__ __forceinline__ void load_window(const Geom &g, const float2 *__restrict__ grid, int grp, int cg0,
                                            const int o[3], int wd[3], float2 *win) {
    const int ns = g.ns;
    int ws[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        wd[d] = d < D ? g.tile[d] + g.W - 1 : 1;
        ws[d] = d < D ? o[d] - (ns - 1) : 0;
    }
    const int wcell = wd[0] * wd[1] * wd[2];
    for (int i = threadIdx.x; i < wcell * CG; i += blockDim.x) {
        const int c = i % CG, w = i / CG;  // coil fastest: consecutive shared-memory words
        const int w2 = w % wd[2], w1 = (w / wd[2]) % wd[1], w0 = w / (wd[2] * wd[1]);
        int gx = (ws[0] + w0) % g.nf[0]; gx += gx < 0 ? g.nf[0] : 0;
        int gy = D > 1 ? (ws[1] + w1) % g.nf[1] : 0; gy += gy < 0 ? g.nf[1] : 0;
        int gz = D > 2 ? (ws[2] + w2) % g.nf[2] : 0; gz += gz < 0 ? g.nf[2] : 0;
        const int coil = cg0 + c;
        float2 val = make_float2(0.f, 0.f);
        if (coil < g.n_coil)
            val = grid[((int64_t)grp * g.n_coil + coil) * g.G + ((int64_t)gx * g.nf[1] + gy) * g.nf[2] + gz];
        win[(size_t)w * CG + c] = val;
    }
}

template <int D, int WT, int CG>
__global__ void __launch_bounds__(512) k_interp(InterpArgs a) {
    extern __shared__ float2 win[];
    const Geom &g = a.g;
    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    int o[3], e[3], wd[3];
    tile_coords<D>(g, sub.x % g.ntiles, o, e);
    load_window<D, CG>(g, a.grid, grp, cg0, o, wd, win);
    __syncthreads();

    const int W = WT ? WT : g.W;
    constexpr int WA = WT ? WT : kMaxW;
    for (int i = threadIdx.x; i < sub.z; i += blockDim.x) {
        const int64_t li = (int64_t)sub.y + i;
        const float4 p = a.pts[li];
        const uint32_t j = a.idx[li];
        int c0[3];
        unpack_cells(D, __float_as_uint(p.w), c0[0], c0[1], c0[2]);
        const float f[3] = {p.x, p.y, p.z};
        float w[D][WA];
        int rel[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < D; ++d) {
            tap_weights<WT>(f[d], g.ns, W, g.beta2[d], w[d]);
            int cc = c0[d] + g.ns - 1;
            if (cc >= g.nf[d]) cc -= g.nf[d];
            rel[d] = cc - o[d];
        }
        float2 acc[CG];
#pragma unroll
        for (int c = 0; c < CG; ++c) acc[c] = make_float2(0.f, 0.f);
        for (int k0 = 0; k0 < W; ++k0) {
            const float w0 = w[0][k0];
            if constexpr (D == 1) {
                const float2 *src = win + (size_t)(rel[0] + k0) * CG;
#pragma unroll
                for (int c = 0; c < CG; ++c) {
                    const float2 s = src[c];
                    acc[c].x = fmaf(w0, s.x, acc[c].x);
                    acc[c].y = fmaf(w0, s.y, acc[c].y);
                }
            } else {
                for (int k1 = 0; k1 < W; ++k1) {
                    const float w01 = w0 * w[1][k1];
                    const size_t row = (size_t)(rel[0] + k0) * wd[1] + rel[1] + k1;
                    if constexpr (D == 2) {
                        const float2 *src = win + row * CG;
#pragma unroll
                        for (int c = 0; c < CG; ++c) {
                            const float2 s = src[c];
                            acc[c].x = fmaf(w01, s.x, acc[c].x);
                            acc[c].y = fmaf(w01, s.y, acc[c].y);
                        }
                    } else {
                        const float2 *src = win + (row * wd[2] + rel[2]) * CG;
#pragma unroll
                        for (int k2 = 0; k2 < WA; ++k2) {
                            if (WT == 0 && k2 >= W) break;
                            const float ww = w01 * w[2][k2];
#pragma unroll
                            for (int c = 0; c < CG; ++c) {
                                const float2 s = src[(size_t)k2 * CG + c];
                                acc[c].x = fmaf(ww, s.x, acc[c].x);
                                acc[c].y = fmaf(ww, s.y, acc[c].y);
                            }
                        }
                    }
                }
            }
        }
        const float sc = a.weight ? a.weight[j] : 1.f;
#pragma unroll
        for (int c = 0; c < CG; ++c) {
            const int coil = cg0 + c;
            if (coil < g.n_coil)
                a.c[(int64_t)j * a.c_elem + (int64_t)coil * a.c_coil] = make_float2(acc[c].x * sc, acc[c].y * sc);
        }
    }
}

// ------------------------------------------------------------------------- gradient
// grad[j, d] = scale * Re( sum_coil conj(gc[j, coil]) * sum_taps F * dw/dx_d ),
// dw/dx = w * (-2 beta d / h) per dimension (analytic derivative of the Gaussian).
template <int D, int WT, int CG>
__global__ void __launch_bounds__(256) k_interp_grad(GradArgs a, float dsc0, float dsc1, float dsc2) {
    extern __shared__ float2 win[];
    const Geom &g = a.g;
    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    int o[3], e[3], wd[3];
    tile_coords<D>(g, sub.x % g.ntiles, o, e);
    load_window<D, CG>(g, a.grid, grp, cg0, o, wd, win);
    __syncthreads();

    const float dsc[3] = {dsc0, dsc1, dsc2};
    const int W = WT ? WT : g.W;
    constexpr int WA = WT ? WT : kMaxW;
    for (int i = threadIdx.x; i < sub.z; i += blockDim.x) {
        const int64_t li = (int64_t)sub.y + i;
        const float4 p = a.pts[li];
        const uint32_t j = a.idx[li];
        int c0[3];
        unpack_cells(D, __float_as_uint(p.w), c0[0], c0[1], c0[2]);
        const float f[3] = {p.x, p.y, p.z};
        float w[D][WA], dw[D][WA];
        int rel[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < D; ++d) {
            tap_weights<WT>(f[d], g.ns, W, g.beta2[d], w[d]);
            const float base = f[d] + (float)(g.ns - 1);
#pragma unroll
            for (int k = 0; k < WA; ++k) {
                if (WT == 0 && k >= W) break;
                dw[d][k] = w[d][k] * dsc[d] * (base - (float)k);
            }
            int cc = c0[d] + g.ns - 1;
            if (cc >= g.nf[d]) cc -= g.nf[d];
            rel[d] = cc - o[d];
        }
        float2 gc[CG];
#pragma unroll
        for (int c = 0; c < CG; ++c) {
            const int coil = cg0 + c;
            gc[c] = coil < g.n_coil ? a.gc[(int64_t)j * a.c_elem + (int64_t)coil * a.c_coil] : make_float2(0.f, 0.f);
        }
        float gd[D];
#pragma unroll
        for (int d = 0; d < D; ++d) gd[d] = 0.f;
        // sum over taps of Re(conj(gc) * F) * dweight, per dimension
        for (int k0 = 0; k0 < W; ++k0) {
            for (int k1 = 0; k1 < (D > 1 ? W : 1); ++k1) {
                for (int k2 = 0; k2 < (D > 2 ? W : 1); ++k2) {
                    size_t cell = rel[0] + k0;
                    if (D > 1) cell = cell * wd[1] + rel[1] + k1;
                    if (D > 2) cell = cell * wd[2] + rel[2] + k2;
                    float re = 0.f;
#pragma unroll
                    for (int c = 0; c < CG; ++c) {
                        const float2 s = win[cell * CG + c];
                        re = fmaf(gc[c].x, s.x, fmaf(gc[c].y, s.y, re));
                    }
                    const float a0 = w[0][k0], a1 = D > 1 ? w[D > 1 ? 1 : 0][k1] : 1.f,
                                a2 = D > 2 ? w[D > 2 ? 2 : 0][k2] : 1.f;
                    gd[0] = fmaf(re, dw[0][k0] * a1 * a2, gd[0]);
                    if (D > 1) gd[D > 1 ? 1 : 0] = fmaf(re, a0 * dw[D > 1 ? 1 : 0][k1] * a2, gd[D > 1 ? 1 : 0]);
                    if (D > 2) gd[D > 2 ? 2 : 0] = fmaf(re, a0 * a1 * dw[D > 2 ? 2 : 0][k2], gd[D > 2 ? 2 : 0]);
                }
            }
        }
#pragma unroll
        for (int d = 0; d < D; ++d) atomicAdd(&a.out[(int64_t)j * D + d], gd[d] * a.scale);
    }
}

}  // namespace gbn
