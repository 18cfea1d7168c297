// 2-D gridding kernels with warp-level accumulation (the multi-coil hot path).
//
// Lane mapping: lane = c + CG*q, coil c in [0, CG), tap slot q in [0, NQ), NQ = 32/CG.
// Slot q handles the y-taps ky = q, q+NQ, q+2NQ, ... (KT of them), so for one grid row a
// warp touches NQ*KT consecutive y cells of CG consecutive coils: with the shared-memory
// layout [x][y][coil] that is one contiguous run of 8-byte words, free of bank conflicts.
//
// Interp: one warp per sample.  Lanes 0..W-1 evaluate wx, lanes 16..16+W-1 evaluate wy
// (one exp2 per lane), shuffles broadcast them, each lane accumulates its KT*W taps for
// its coil, and a shuffle reduction over the NQ slots yields the coil value.
//
// Spread: output-stationary tile [TX][TY][CG] in shared memory; warp w owns tile rows
// [w*R, (w+1)*R).  A batch of samples is staged (weights, coil values, local offsets),
// then every warp walks the batch and applies the taps that fall in its own rows.  No
// two warps ever write the same cell and the lanes of a warp write distinct cells, so the
// accumulation is plain load-add-store: no atomics, and a fixed summation order.
#pragma once

#include "common.cuh"

namespace gbn {

template <int WT, int CG>
struct Lanes2D {
    static constexpr int NQ = 32 / CG;
    static constexpr int WMAX = WT ? WT : 16;
    static constexpr int KT = (WMAX + NQ - 1) / NQ;
};

__device__ __forceinline__ int wrap_mod(int v, int n) {
    v %= n;
    return v < 0 ? v + n : v;
}

// v in [-n, inf): wrapped into [0, n) without a division (the loop runs only when a window
// is wider than the grid)
__device__ __forceinline__ int wrap_fast(int v, int n) {
    v += v < 0 ? n : 0;
    while (v >= n) v -= n;
    return v;
}

// a / b for 0 <= a < 2^20 and 1 <= b, with rb = 1.0f / b: (a + 0.5) * rb is within
// 2^-21 (a/b) of the true quotient, far less than the 0.5/b to the nearest integer
__device__ __forceinline__ int div_small(int a, float rb) { return (int)(((float)a + 0.5f) * rb); }

// --------------------------------------------------------------------------------- interp
template <int WT, int CG>
__global__ void __launch_bounds__(512) k_interp2d(InterpArgs a) {
    using L = Lanes2D<WT, CG>;
    extern __shared__ float4 smem_i2[];
    float2 *win = reinterpret_cast<float2 *>(smem_i2);  // [WX][WY][CG]
    const Geom &g = a.g;
    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    const int tile = sub.x % g.ntiles;
    const int o0 = (tile / g.ntile[1]) * g.tile[0];
    const int o1 = (tile % g.ntile[1]) * g.tile[1];
    const int W = WT ? WT : g.W;
    const int ns = g.ns;
    const int WX = g.tile[0] + W - 1, WY = g.tile[1] + W - 1;
    const int nf0 = g.nf[0], nf1 = g.nf[1];

    // stage the window (periodic wrap), all CG coils of a cell contiguous; coil fastest
    // across threads, so the shared-memory stores are consecutive 8-byte words and each
    // warp's global loads are CG runs of 32/CG consecutive cells
    {
        const int ws0 = o0 - (ns - 1), ws1 = o1 - (ns - 1);
        const float2 *base = a.grid + ((int64_t)grp * g.n_coil + cg0) * g.G;
        const int nitem = WX * WY * CG;
        const float rWY = 1.f / (float)WY;
        for (int i = threadIdx.x; i < nitem; i += blockDim.x) {
            const int c = i % CG, cell = i / CG;  // CG is a power of two
            const int wx = div_small(cell, rWY), wy = cell - wx * WY;
            const int gx = wrap_fast(ws0 + wx, nf0), gy = wrap_fast(ws1 + wy, nf1);
            win[i] = (cg0 + c < g.n_coil) ? base[(int64_t)c * g.G + (int64_t)gx * nf1 + gy] : make_float2(0.f, 0.f);
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int c = lane % CG, q = lane / CG;
    const int kk = lane & 15;
    const float beta = lane < 16 ? g.beta2[0] : g.beta2[1];
    // software pipeline: the next sample's record is in flight while this one is gathered
    float4 p_next = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t j_next = 0;
    if (warp < sub.z) {
        p_next = a.pts[(int64_t)sub.y + warp];
        j_next = a.idx[(int64_t)sub.y + warp];
    }
    for (int s = warp; s < sub.z; s += nw) {
        const float4 p = p_next;
        const uint32_t j = j_next;
        if (s + nw < sub.z) {
            p_next = a.pts[(int64_t)sub.y + s + nw];
            j_next = a.idx[(int64_t)sub.y + s + nw];
        }
        int c0x, c0y, c0z;
        unpack_cells(2, __float_as_uint(p.w), c0x, c0y, c0z);
        int ccx = c0x + ns - 1, ccy = c0y + ns - 1;
        ccx -= ccx >= nf0 ? nf0 : 0;
        ccy -= ccy >= nf1 ? nf1 : 0;
        const int rel0 = ccx - o0, rel1 = ccy - o1;
        float myw = 0.f;
        if (kk < W) {
            const float d = (lane < 16 ? p.x : p.y) + (float)(ns - 1 - kk);
            myw = exp2f(-beta * d * d);
        }
        float wy[L::KT];
#pragma unroll
        for (int t = 0; t < L::KT; ++t) {
            const int ky = q + t * L::NQ;
            const float v = __shfl_sync(0xffffffffu, myw, 16 + (ky < 16 ? ky : 15));
            wy[t] = ky < W ? v : 0.f;
        }
        // a lane's y taps are fixed, so it sums wx * G over x per tap slot and applies its
        // y weights once at the end: one load and one packed FMA per tap
        float2 acc[L::KT];
#pragma unroll
        for (int t = 0; t < L::KT; ++t) acc[t] = make_float2(0.f, 0.f);
        const float2 *rowbase = win + ((size_t)rel0 * WY + rel1) * CG + c;
#pragma unroll
        for (int kx = 0; kx < L::WMAX; ++kx) {
            if (WT == 0 && kx >= W) break;
            const float wx = __shfl_sync(0xffffffffu, myw, kx);
            const float2 wx2 = make_float2(wx, wx);
            const float2 *row = rowbase + (size_t)kx * WY * CG;
#pragma unroll
            for (int t = 0; t < L::KT; ++t) {
                const int ky = q + t * L::NQ;
                if (ky < W) acc[t] = __ffma2_rn(wx2, row[ky * CG], acc[t]);
            }
        }
        float ax = 0.f, ay = 0.f;
#pragma unroll
        for (int t = 0; t < L::KT; ++t) {
            ax = fmaf(wy[t], acc[t].x, ax);
            ay = fmaf(wy[t], acc[t].y, ay);
        }
#pragma unroll
        for (int off = CG; off < 32; off <<= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, off);
            ay += __shfl_xor_sync(0xffffffffu, ay, off);
        }
        if (q == 0 && cg0 + c < g.n_coil) {
            const float sc = a.weight ? a.weight[j] : 1.f;
            a.c[(int64_t)j * a.c_elem + (int64_t)(cg0 + c) * a.c_coil] = make_float2(ax * sc, ay * sc);
        }
    }
}

// --------------------------------------------------------------------------------- spread
constexpr int kSpreadBatch = 64;  // samples staged per batch

template <int WT, int CG>
__global__ void __launch_bounds__(512) k_spread2d(SpreadArgs a) {
    using L = Lanes2D<WT, CG>;
    extern __shared__ float4 smem_s2[];
    const Geom &g = a.g;
    const int TX = g.tile[0], TY = g.tile[1];
    float2 *acc = reinterpret_cast<float2 *>(smem_s2);              // [TX][TY][CG]
    float *st_w = reinterpret_cast<float *>(acc + (size_t)TX * TY * CG);  // [batch][32]: wx[16], wy[16]
    float2 *st_v = reinterpret_cast<float2 *>(st_w + kSpreadBatch * 32);  // [batch][CG]
    int2 *st_r = reinterpret_cast<int2 *>(st_v + kSpreadBatch * CG);      // [batch]: local first-tap cell
    int *st_y = reinterpret_cast<int *>(st_r + kSpreadBatch);             // [batch][16]: local y of tap ky, -1 off tile

    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    const int tile = sub.x % g.ntiles;
    const int o0 = (tile / g.ntile[1]) * TX;
    const int o1 = (tile % g.ntile[1]) * TY;
    const int nf0 = g.nf[0], nf1 = g.nf[1];
    const int e0 = min(TX, nf0 - o0), e1 = min(TY, nf1 - o1);
    const int W = WT ? WT : g.W;
    const int ns = g.ns;

    for (int i = threadIdx.x; i < TX * TY * CG; i += blockDim.x) acc[i] = make_float2(0.f, 0.f);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int c = lane % CG, q = lane / CG;
    const int R = (TX + nw - 1) / nw;
    const int row0 = warp * R, row1 = min(row0 + R, e0);

    for (int base = 0; base < sub.z; base += kSpreadBatch) {
        const int n = min(kSpreadBatch, sub.z - base);
        __syncthreads();  // previous batch consumed (and the zeroing above done)
        for (int i = threadIdx.x; i < n * 32; i += blockDim.x) {
            const int s = i >> 5, k = i & 31, kq = k & 15;
            const float4 p = a.pts[(int64_t)sub.y + base + s];
            float val = 0.f;
            if (kq < W) {
                const float d = (k < 16 ? p.x : p.y) + (float)(ns - 1 - kq);
                val = exp2f(-(k < 16 ? g.beta2[0] : g.beta2[1]) * d * d);
            }
            st_w[i] = val;
            // signed local position of the first tap: in (-W, nf - W].  The stencil
            // [r, r + W) never wraps onto the tile twice because nf >= tile + W on this
            // path (the generic kernel serves smaller grids).
            int c0x, c0y, c0z;
            unpack_cells(2, __float_as_uint(p.w), c0x, c0y, c0z);
            int rx = c0x - o0, ry = c0y - o1;
            rx += rx < 0 ? nf0 : 0;
            ry += ry < 0 ? nf1 : 0;
            rx -= rx > nf0 - W ? nf0 : 0;
            ry -= ry > nf1 - W ? nf1 : 0;
            if (k == 0) st_r[s] = make_int2(rx, ry);
            if (k >= 16) {
                const int y = ry + kq;
                st_y[s * 16 + kq] = (kq < W && (unsigned)y < (unsigned)e1) ? y : -1;
            }
        }
        for (int i = threadIdx.x; i < n * CG; i += blockDim.x) {
            const int s = i / CG, cc = i - s * CG;
            const int64_t li = (int64_t)sub.y + base + s;
            const uint32_t j = a.idx[li];
            float2 v = make_float2(0.f, 0.f);
            if (cg0 + cc < g.n_coil) {
                v = a.c[(int64_t)j * a.c_elem + (int64_t)(cg0 + cc) * a.c_coil];
                if (a.weight) {
                    const float sw = a.weight[j];
                    v.x *= sw;
                    v.y *= sw;
                }
            }
            st_v[i] = v;
        }
        __syncthreads();

        for (int s = 0; s < n; ++s) {
            const int2 r = st_r[s];
            // rows of this warp that the stencil [r.x, r.x + W) reaches
            const int lo = max(row0, r.x), hi = min(row1, r.x + W);
            if (lo >= hi) continue;
            const float2 v = st_v[s * CG + c];
            const float *w = st_w + s * 32;
            if constexpr (CG == 1) {
                // one coil: lane (xo, ky) takes y tap ky on every other row from lo + xo, so
                // 32 lanes cover 16 tap slots on two rows at once
                const int ky = lane & 15, xo = lane >> 4;
                const int yy = st_y[s * 16 + ky];
                const float wy = w[16 + ky];
                const float2 wyv1 = make_float2(wy * v.x, wy * v.y);
                const float *wx_row1 = w - r.x;
                float2 *dst1 = acc + (size_t)(lo + xo) * TY + yy;
#pragma unroll 4
                for (int row = lo + xo; row < hi; row += 2, dst1 += 2 * TY) {
                    const float wx = wx_row1[row];
                    if (yy >= 0) *dst1 = __ffma2_rn(make_float2(wx, wx), wyv1, *dst1);
                }
            } else {
                // per lane: the column weight folded into the coil value, and the tap's tile column
                float2 wyv[L::KT];
                int ly[L::KT];
#pragma unroll
                for (int t = 0; t < L::KT; ++t) {
                    const int ky = q + t * L::NQ;
                    const bool in = ky < 16;
                    const float wy = in ? w[16 + (in ? ky : 0)] : 0.f;
                    ly[t] = in ? st_y[s * 16 + (in ? ky : 0)] : -1;
                    wyv[t] = make_float2(wy * v.x, wy * v.y);
                }
                const float *wx_row = w - r.x;
                float2 *dst = acc + (size_t)lo * TY * CG + c;
#pragma unroll 4
                for (int row = lo; row < hi; ++row, dst += TY * CG) {
                    const float wx = wx_row[row];
                    const float2 wx2 = make_float2(wx, wx);
#pragma unroll
                    for (int t = 0; t < L::KT; ++t) {
                        if (ly[t] >= 0) {
                            float2 *cell = dst + (size_t)ly[t] * CG;
                            *cell = __ffma2_rn(wx2, wyv[t], *cell);
                        }
                    }
                }
            }
        }
    }
    __syncthreads();

    // flush: consecutive threads take consecutive coils of a cell (shared reads contiguous,
    // each coil plane receives 32-byte runs)
    const bool split = (sub.w & kSplitFlag) != 0;
    const int ecell = e0 * e1;
    for (int i = threadIdx.x; i < ecell * CG; i += blockDim.x) {
        const int cc = i % CG, cell = i / CG;
        if (cg0 + cc >= g.n_coil) continue;
        const int lx = cell / e1, ly = cell - lx * e1;
        const float2 val = acc[((size_t)lx * TY + ly) * CG + cc];
        float2 *dst = a.grid + ((int64_t)grp * g.n_coil + cg0 + cc) * g.G + (int64_t)(o0 + lx) * nf1 + (o1 + ly);
        if (split) {
            atomicAdd(&dst->x, val.x);
            atomicAdd(&dst->y, val.y);
        } else {
            *dst = val;
        }
    }
}

// ------------------------------------------------------------------ spread, register tile
// For 4 or 8 coils per block the output tile lives in registers: warp w owns the rows
// [4w, 4w + 4) and lane (c, q) holds columns q, q + NQ, q + 2NQ, q + 3NQ of coil c, so the
// tile is (4 * warps) x (4 * NQ) cells.  There is no shared-memory read-modify-write.
//
// Samples are staged in double-buffered batches of 32 (one barrier per batch).  Warp 0
// stages the x weight of every tile row for each sample (0 outside the stencil) and builds,
// with ballots, the ordered list of samples whose stencil reaches each warp's rows; warp 1
// stages the y weight of every tile column, stored [q][k] for column q + k*NQ so a lane
// reads its 4 columns with one 16-byte load; the other warps gather the coil values.  A
// warp then walks only its own list: per sample one load of its 4 row weights, one of its
// 4 column weights, the coil value, 8 multiplies and 16 packed FMAs.  The summation order
// is the sample order, fixed for a given trajectory.
constexpr int kRegRows = 4;    // rows per warp
constexpr int kRegCols = 4;    // columns per lane
constexpr int kRegBatch = 32;  // samples per staged batch

// Stride (floats) of a staged per-sample weight row of n floats: a multiple of 4 for
// 16-byte loads and stores, and an odd number of 16-byte units so that the 16-byte stores
// of 8 consecutive lanes fill the 32 banks exactly once (conflict-free staging).
__host__ __device__ inline int reg_stride(int n) {
    int n4 = (n + 3) / 4;
    n4 += (n4 % 2 == 0) ? 1 : 0;
    return 4 * n4;
}

__device__ __forceinline__ unsigned lanemask_lt(int lane) { return (1u << lane) - 1u; }

// Gaussian weight of tap `tap` (0 outside [0, W)) for in-cell fraction f
__device__ __forceinline__ float tap_weight(bool ok, int tap, int W, float f, int ns, float beta2) {
    if (!ok || (unsigned)tap >= (unsigned)W) return 0.f;
    const float d = f + (float)(ns - 1 - tap);
    return exp2f(-beta2 * d * d);
}

template <int WT, int CG>
__global__ void __launch_bounds__(256) k_spread2d_reg(SpreadArgs a) {
    constexpr int NQ = 32 / CG;
    constexpr int B = kRegBatch;
    extern __shared__ float4 smem_r2[];
    const Geom &g = a.g;
    const int TX = g.tile[0], TY = g.tile[1];  // TX = 4 * warps, TY = 4 * NQ (set by the host)
    const int TXP = reg_stride(TX), TYP = reg_stride(TY);
    const int nw = blockDim.x >> 5;
    float *st_wr = reinterpret_cast<float *>(smem_r2);                     // [2][B][TXP]
    float *st_wc = st_wr + 2 * B * TXP;                                    // [2][B][TYP]: [q][k]
    float2 *st_v = reinterpret_cast<float2 *>(st_wc + 2 * B * TYP);        // [2][B][CG]
    int *st_cnt = reinterpret_cast<int *>(st_v + 2 * B * CG);              // [2][8]
    uint8_t *st_list = reinterpret_cast<uint8_t *>(st_cnt + 16);           // [2][8][B]

    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    const int tile = sub.x % g.ntiles;
    const int o0 = (tile / g.ntile[1]) * TX;
    const int o1 = (tile % g.ntile[1]) * TY;
    const int nf0 = g.nf[0], nf1 = g.nf[1];
    const int e0 = min(TX, nf0 - o0), e1 = min(TY, nf1 - o1);
    const int W = WT ? WT : g.W;
    const int ns = g.ns;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = lane % CG, q = lane / CG;
    const int row0 = warp * kRegRows;
    float2 acc[kRegRows][kRegCols];
#pragma unroll
    for (int r = 0; r < kRegRows; ++r)
#pragma unroll
        for (int k = 0; k < kRegCols; ++k) acc[r][k] = make_float2(0.f, 0.f);

    for (int base = 0, buf = 0; base < sub.z; base += B, buf ^= 1) {
        const int n = min(B, sub.z - base);
        if (warp < 2) {
            // warp 0: row weights and the per-warp lists; warp 1: column weights
            const bool ok = lane < n;
            int rx = 0, ry = 0;
            float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
            if (ok) {
                p = a.pts[(int64_t)sub.y + base + lane];
                // signed local first-tap cell, in (-W, nf - W] (nf >= tile + W on this path)
                int c0x, c0y, c0z;
                unpack_cells(2, __float_as_uint(p.w), c0x, c0y, c0z);
                rx = c0x - o0;
                ry = c0y - o1;
                rx += rx < 0 ? nf0 : 0;
                ry += ry < 0 ? nf1 : 0;
                rx -= rx > nf0 - W ? nf0 : 0;
                ry -= ry > nf1 - W ? nf1 : 0;
            }
            if (warp == 0) {
                float *dst = st_wr + (buf * B + lane) * TXP;
                for (int r4 = 0; r4 < TX; r4 += 4) {
                    const float b = g.beta2[0];
                    *reinterpret_cast<float4 *>(dst + r4) =
                        make_float4(tap_weight(ok, r4 - rx, W, p.x, ns, b), tap_weight(ok, r4 + 1 - rx, W, p.x, ns, b),
                                    tap_weight(ok, r4 + 2 - rx, W, p.x, ns, b), tap_weight(ok, r4 + 3 - rx, W, p.x, ns, b));
                }
                for (int w = 0; w < nw; ++w) {
                    const bool hit = ok && rx < w * kRegRows + kRegRows && rx + W > w * kRegRows;
                    const unsigned m = __ballot_sync(0xffffffffu, hit);
                    if (hit) st_list[(buf * 8 + w) * B + __popc(m & lanemask_lt(lane))] = (uint8_t)lane;
                    if (lane == 0) st_cnt[buf * 8 + w] = __popc(m);
                }
            } else {
                float *dst = st_wc + (buf * B + lane) * TYP;
                const float b = g.beta2[1];
#pragma unroll
                for (int cq = 0; cq < NQ; ++cq)  // columns cq + k*NQ, k = 0..3, as one 16-byte store
                    *reinterpret_cast<float4 *>(dst + cq * 4) =
                        make_float4(tap_weight(ok, cq - ry, W, p.y, ns, b), tap_weight(ok, cq + NQ - ry, W, p.y, ns, b),
                                    tap_weight(ok, cq + 2 * NQ - ry, W, p.y, ns, b),
                                    tap_weight(ok, cq + 3 * NQ - ry, W, p.y, ns, b));
            }
        } else {
            for (int i = threadIdx.x - 64; i < n * CG; i += blockDim.x - 64) {
                const int s = i / CG, cc = i - s * CG;
                const uint32_t j = a.idx[(int64_t)sub.y + base + s];
                float2 v = make_float2(0.f, 0.f);
                if (cg0 + cc < g.n_coil) {
                    v = a.c[(int64_t)j * a.c_elem + (int64_t)(cg0 + cc) * a.c_coil];
                    if (a.weight) {
                        const float sw = a.weight[j];
                        v.x *= sw;
                        v.y *= sw;
                    }
                }
                st_v[buf * B * CG + i] = v;
            }
        }
        // the other buffer was last read before this barrier's previous instance, so one
        // barrier per batch suffices
        __syncthreads();

        const int cnt = st_cnt[buf * 8 + warp];
        const uint8_t *lst = st_list + (buf * 8 + warp) * B;
        for (int i = 0; i < cnt; ++i) {
            const int s = buf * B + lst[i];
            const float4 wc = *reinterpret_cast<const float4 *>(st_wc + s * TYP + q * 4);
            const float4 wr = *reinterpret_cast<const float4 *>(st_wr + s * TXP + row0);
            const float2 v = st_v[s * CG + c];
            const float2 u[kRegCols] = {make_float2(wc.x * v.x, wc.x * v.y), make_float2(wc.y * v.x, wc.y * v.y),
                                        make_float2(wc.z * v.x, wc.z * v.y), make_float2(wc.w * v.x, wc.w * v.y)};
            const float wrr[kRegRows] = {wr.x, wr.y, wr.z, wr.w};
#pragma unroll
            for (int rr = 0; rr < kRegRows; ++rr) {
                const float2 wx2 = make_float2(wrr[rr], wrr[rr]);
#pragma unroll
                for (int k = 0; k < kRegCols; ++k) acc[rr][k] = __ffma2_rn(wx2, u[k], acc[rr][k]);
            }
        }
    }

    // flush the register tile: rows and columns beyond the grid edge are dropped
    if (cg0 + c >= g.n_coil) return;
    const bool split = (sub.w & kSplitFlag) != 0;
    float2 *dstc = a.grid + ((int64_t)grp * g.n_coil + cg0 + c) * g.G;
#pragma unroll
    for (int rr = 0; rr < kRegRows; ++rr) {
        const int lx = row0 + rr;
        if (lx >= e0) break;
#pragma unroll
        for (int k = 0; k < kRegCols; ++k) {
            const int ly = q + k * NQ;
            if (ly >= e1) continue;
            float2 *dst = dstc + (int64_t)(o0 + lx) * nf1 + (o1 + ly);
            if (split) {
                atomicAdd(&dst->x, acc[rr][k].x);
                atomicAdd(&dst->y, acc[rr][k].y);
            } else {
                *dst = acc[rr][k];
            }
        }
    }
}

inline size_t spread2d_reg_smem_bytes(const Geom &g, int cg) {
    return 2 * ((size_t)kRegBatch * (reg_stride(g.tile[0]) + reg_stride(g.tile[1])) * sizeof(float) +
                (size_t)kRegBatch * cg * sizeof(float2)) +
           16 * sizeof(int) + 2 * 8 * kRegBatch;
}

inline size_t spread2d_smem_bytes(const Geom &g, int cg) {
    return (size_t)g.tile[0] * g.tile[1] * cg * sizeof(float2) + kSpreadBatch * 32 * sizeof(float) +
           (size_t)kSpreadBatch * cg * sizeof(float2) + kSpreadBatch * sizeof(int2) +
           kSpreadBatch * 16 * sizeof(int);
}

inline size_t interp2d_smem_bytes(const Geom &g, int cg) {
    return (size_t)(g.tile[0] + g.W - 1) * (g.tile[1] + g.W - 1) * cg * sizeof(float2);
}

// ----------------------------------------------------------------- trajectory gradient, 2-D
// grad_x[j, d] += scale * Re( sum_coil conj(gc[j, coil]) dc_j/dx_d ) with
// dc/dx_0 = sum dwx[kx] wy[ky] G and dc/dx_1 = sum wx[kx] dwy[ky] G, dw = w * dsc * dist
// (the analytic derivative of the Gaussian weight at tap distance dist, in cells).  The
// k_interp2d sample loop with two sums per tap slot: b += dwx G and a += wx G; the y weights
// and their derivatives are applied once per slot, then the slots, and after weighting with
// the upstream gradient the coils, are reduced by shuffles.  The window is staged as in
// k_interp2d ([x][y][coil]).
template <int WT, int CG>
__global__ void __launch_bounds__(512) k_interp_grad2d(GradArgs a, float dsc0, float dsc1) {
    using L = Lanes2D<WT, CG>;
    extern __shared__ float4 smem_g2[];
    float2 *win = reinterpret_cast<float2 *>(smem_g2);  // [WX][WY][CG]
    const Geom &g = a.g;
    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    const int tile = sub.x % g.ntiles;
    const int o0 = (tile / g.ntile[1]) * g.tile[0];
    const int o1 = (tile % g.ntile[1]) * g.tile[1];
    const int W = WT ? WT : g.W;
    const int ns = g.ns;
    const int WX = g.tile[0] + W - 1, WY = g.tile[1] + W - 1;
    const int nf0 = g.nf[0], nf1 = g.nf[1];
    {
        const int ws0 = o0 - (ns - 1), ws1 = o1 - (ns - 1);
        const float2 *base = a.grid + ((int64_t)grp * g.n_coil + cg0) * g.G;
        const int nitem = WX * WY * CG;
        const float rWY = 1.f / (float)WY;
        for (int i = threadIdx.x; i < nitem; i += blockDim.x) {
            const int c = i % CG, cell = i / CG;
            const int wx = div_small(cell, rWY), wy = cell - wx * WY;
            const int gx = wrap_fast(ws0 + wx, nf0), gy = wrap_fast(ws1 + wy, nf1);
            win[i] = (cg0 + c < g.n_coil) ? base[(int64_t)c * g.G + (int64_t)gx * nf1 + gy] : make_float2(0.f, 0.f);
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int c = lane % CG, q = lane / CG;
    const int kk = lane & 15;
    const float beta = lane < 16 ? g.beta2[0] : g.beta2[1];
    const float dsc = lane < 16 ? dsc0 : dsc1;
    for (int s = warp; s < sub.z; s += nw) {
        const float4 p = a.pts[(int64_t)sub.y + s];
        const uint32_t j = a.idx[(int64_t)sub.y + s];
        int c0x, c0y, c0z;
        unpack_cells(2, __float_as_uint(p.w), c0x, c0y, c0z);
        int ccx = c0x + ns - 1, ccy = c0y + ns - 1;
        ccx -= ccx >= nf0 ? nf0 : 0;
        ccy -= ccy >= nf1 ? nf1 : 0;
        const int rel0 = ccx - o0, rel1 = ccy - o1;
        float myw = 0.f, mydw = 0.f;
        if (kk < W) {
            const float d = (lane < 16 ? p.x : p.y) + (float)(ns - 1 - kk);
            myw = exp2f(-beta * d * d);
            mydw = myw * dsc * d;
        }
        float wy[L::KT], dwy[L::KT];
#pragma unroll
        for (int t = 0; t < L::KT; ++t) {
            const int ky = q + t * L::NQ;
            const int src = 16 + (ky < 16 ? ky : 15);
            const float v = __shfl_sync(0xffffffffu, myw, src), dv = __shfl_sync(0xffffffffu, mydw, src);
            wy[t] = ky < W ? v : 0.f;
            dwy[t] = ky < W ? dv : 0.f;
        }
        float2 sa[L::KT], sb[L::KT];
#pragma unroll
        for (int t = 0; t < L::KT; ++t) {
            sa[t] = make_float2(0.f, 0.f);
            sb[t] = make_float2(0.f, 0.f);
        }
        const float2 *rowbase = win + ((size_t)rel0 * WY + rel1) * CG + c;
#pragma unroll
        for (int kx = 0; kx < L::WMAX; ++kx) {
            if (WT == 0 && kx >= W) break;
            const float wx = __shfl_sync(0xffffffffu, myw, kx), dwx = __shfl_sync(0xffffffffu, mydw, kx);
            const float2 wx2 = make_float2(wx, wx), dwx2 = make_float2(dwx, dwx);
            const float2 *row = rowbase + (size_t)kx * WY * CG;
#pragma unroll
            for (int t = 0; t < L::KT; ++t) {
                const int ky = q + t * L::NQ;
                if (ky < W) {
                    const float2 G = row[ky * CG];
                    sa[t] = __ffma2_rn(wx2, G, sa[t]);
                    sb[t] = __ffma2_rn(dwx2, G, sb[t]);
                }
            }
        }
        float gx_re = 0.f, gx_im = 0.f, gy_re = 0.f, gy_im = 0.f;
#pragma unroll
        for (int t = 0; t < L::KT; ++t) {
            gx_re = fmaf(wy[t], sb[t].x, gx_re);
            gx_im = fmaf(wy[t], sb[t].y, gx_im);
            gy_re = fmaf(dwy[t], sa[t].x, gy_re);
            gy_im = fmaf(dwy[t], sa[t].y, gy_im);
        }
#pragma unroll
        for (int off = CG; off < 32; off <<= 1) {
            gx_re += __shfl_xor_sync(0xffffffffu, gx_re, off);
            gx_im += __shfl_xor_sync(0xffffffffu, gx_im, off);
            gy_re += __shfl_xor_sync(0xffffffffu, gy_re, off);
            gy_im += __shfl_xor_sync(0xffffffffu, gy_im, off);
        }
        // Re(conj(gc) * dc/dx) per coil (slot-0 lanes), then summed over the coils
        float g0 = 0.f, g1 = 0.f;
        if (q == 0 && cg0 + c < g.n_coil) {
            const float2 gc = a.gc[(int64_t)j * a.c_elem + (int64_t)(cg0 + c) * a.c_coil];
            g0 = gc.x * gx_re + gc.y * gx_im;
            g1 = gc.x * gy_re + gc.y * gy_im;
        }
#pragma unroll
        for (int off = 1; off < CG; off <<= 1) {
            g0 += __shfl_xor_sync(0xffffffffu, g0, off);
            g1 += __shfl_xor_sync(0xffffffffu, g1, off);
        }
        if (lane == 0) {
            atomicAdd(&a.out[(int64_t)j * 2], g0 * a.scale);
            atomicAdd(&a.out[(int64_t)j * 2 + 1], g1 * a.scale);
        }
    }
}

}  // namespace gbn
