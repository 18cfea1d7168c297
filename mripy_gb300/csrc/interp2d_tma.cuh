// 2-D interp with grid windows staged by TMA (the forward direction's hot kernel).
//
// Persistent blocks walk the work items (interp subproblem x coil group) with a stride of
// the grid size.  Each item needs the window of its home bin: (tile + W - 1) cells per
// dimension around the bin, CG coils.  For bins whose window lies inside the grid one
// elected thread loads it with a single 3-D tensor copy (cp.async.bulk.tensor: box
// BY x BX x CG of 8-byte cells, y innermost) that completes on an mbarrier; windows that
// wrap around the periodic grid edge are gathered by all threads with ordinary loads.
// A ring of S window buffers (2 to 4, as many as fit the shared-memory budget) holds the
// block's next S items: the copy for item k + S is issued as soon as item k's buffer is
// released, so a block computes on one window while the next S - 1 are in flight.  The
// issuing thread also leaves the item's decoded geometry beside its buffer.  Waits
// suspend the threads in hardware (mbarrier.try_wait) instead of spinning.
//
// Shared-memory layout per buffer: [coil][x][y] with row pitch BY and coil stride
// CS = BX * BY, exactly the order the tensor copy writes.  BX, BY are chosen on the host
// so that a warp's reads (CG coils x 32/CG consecutive y cells) fall on distinct banks.
// The box's inner extent BY is even and its y start is rounded down to an even cell
// (16-byte boundary), so the window may start one cell into the row (off1).
//
// Every mbarrier wait is bounded: after kTmaWaitLimit polls the block records
// kStatusTmaTimeout in the plan's status word (read by gbn_plan_status) and goes on, so
// no launch can hang.  The sample loop is the k_interp2d one (warp per sample, lanes =
// coils x tap slots, per-slot sums of wx * G, y weights applied once).
#pragma once

#include <cuda.h>

#include "grid2d_kernels.cuh"
#include "tma.cuh"

namespace gbn {

constexpr int kTmaMaxStages = 4;              // window buffers per block (ring)

struct TmaItem {
    int4 sub;
    int grp, cg0, o0, o1, ws0, ws1, ys;
    bool tma;  // the window lies inside the grid: one box copy
};

template <int CG>
__device__ __forceinline__ TmaItem tma_item(const InterpArgs &a, const TmaWin &t, int64_t item) {
    const Geom &g = a.g;
    TmaItem r;
    const int64_t si = item / t.n_cg;
    r.cg0 = (int)(item - si * t.n_cg) * CG * t.passes;
    r.sub = a.subs[si];
    r.grp = r.sub.x / g.ntiles;
    const int tile = r.sub.x % g.ntiles;
    r.o0 = (tile / g.ntile[1]) * g.tile[0];
    r.o1 = (tile % g.ntile[1]) * g.tile[1];
    r.ws0 = r.o0 - (g.ns - 1);
    r.ws1 = r.o1 - (g.ns - 1);
    r.ys = r.ws1 - (r.ws1 & 1);  // even y start (16-byte boundary); used only when ws1 >= 0
    r.tma = r.ws0 >= 0 && r.ws0 + t.BX <= g.nf[0] && r.ws1 >= 0 && r.ys + t.BY <= g.nf[1];
    return r;
}

template <int CG>
__device__ __forceinline__ void tma_issue(const InterpArgs &a, const TmaWin &t, const CUtensorMap *map,
                                          const TmaItem &it, float2 *buf, uint64_t *bar) {
    fence_proxy_async_smem();  // the buffer's previous readers are ordered before the copy
    mbar_arrive_expect_tx(bar, t.box_bytes);
    tma_load_3d(buf, map, it.ys, it.ws0, it.grp * a.g.n_coil + it.cg0, bar);
}

// MULTI: items hold several coil groups (t.passes > 1); the single-group instance keeps
// fewer registers (x weights shuffled per tap row instead of kept).
template <int WT, int CG, bool MULTI>
__global__ void __launch_bounds__(512) k_interp2d_tma(InterpArgs a, const __grid_constant__ CUtensorMap map,
                                                      TmaWin t, uint32_t *status) {
    using L = Lanes2D<WT, CG>;
    extern __shared__ __align__(128) float4 smem_t2[];
    float2 *bufs = reinterpret_cast<float2 *>(smem_t2);  // [stages][buf_elems]
    __shared__ __align__(8) uint64_t bar[kTmaMaxStages];
    __shared__ TmaItem ring[kTmaMaxStages];  // geometry of the item each buffer holds / awaits
    const Geom &g = a.g;
    const int W = WT ? WT : g.W;
    const int ns = g.ns;
    const int WX = g.tile[0] + W - 1, WY = g.tile[1] + W - 1;
    const int nf0 = g.nf[0], nf1 = g.nf[1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int c = lane % CG, q = lane / CG;
    const int kk = lane & 15;
    const float beta = lane < 16 ? g.beta2[0] : g.beta2[1];
    const int64_t stride = gridDim.x;
    const int S = t.stages;

    if (threadIdx.x == 0) {
        for (int b = 0; b < S; ++b) mbar_init(&bar[b], 1);
        fence_barrier_init();
        // prologue: the first S items of this block (box copies where the window is inside)
        for (int b = 0; b < S; ++b) {
            const int64_t item = blockIdx.x + b * stride;
            if (item < t.n_items) {
                ring[b] = tma_item<CG>(a, t, item);
                if (ring[b].tma) tma_issue<CG>(a, t, &map, ring[b], bufs + (size_t)b * t.buf_elems, &bar[b]);
            }
        }
    }
    __syncthreads();

    uint32_t parity = 0u;  // bit b: phase parity expected next on buffer b's barrier
    int b = 0;
    for (int64_t item = blockIdx.x; item < t.n_items; item += stride, b = (b + 1 == S) ? 0 : b + 1) {
        float2 *win = bufs + (size_t)b * t.buf_elems;
        const TmaItem it = ring[b];
        int off1 = 0;
        if (it.tma) {
            if (!mbar_wait_bounded(&bar[b], (parity >> b) & 1u) && lane == 0) atomicOr(status, kStatusTmaTimeout);
            parity ^= 1u << b;
            off1 = it.ws1 - it.ys;
        } else {
            // the window wraps: gather it with periodic indices, y fastest (coalesced)
            const float2 *base = a.grid + ((int64_t)it.grp * g.n_coil + it.cg0) * g.G;
            const int n = CG * t.passes * WX * WY;
            const float rWY = 1.f / (float)WY, rWX = 1.f / (float)WX;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int row = div_small(i, rWY), wy = i - row * WY;
                const int cc = div_small(row, rWX), wx = row - cc * WX;
                const int gx = wrap_fast(it.ws0 + wx, nf0), gy = wrap_fast(it.ws1 + wy, nf1);
                win[cc * t.CS + wx * t.BY + wy] = (it.cg0 + cc < g.n_coil)
                                                      ? base[(int64_t)cc * g.G + (int64_t)gx * nf1 + gy]
                                                      : make_float2(0.f, 0.f);
            }
            __syncthreads();
        }

        const int4 sub = it.sub;
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
            const int rel0 = ccx - it.o0, rel1 = ccy - it.o1;
            float myw = 0.f;
            if (kk < W) {
                const float d = (lane < 16 ? p.x : p.y) + (float)(ns - 1 - kk);
                myw = exp2f(-beta * d * d);
            }
            float wy[L::KT];
#pragma unroll
            for (int tt = 0; tt < L::KT; ++tt) {
                const int ky = q + tt * L::NQ;
                const float v = __shfl_sync(0xffffffffu, myw, 16 + (ky < 16 ? ky : 15));
                wy[tt] = ky < W ? v : 0.f;
            }
            float wxs[MULTI ? L::WMAX : 1];  // MULTI: x weights kept for every coil pass
            if constexpr (MULTI) {
#pragma unroll
                for (int kx = 0; kx < L::WMAX; ++kx) wxs[kx] = __shfl_sync(0xffffffffu, myw, kx);
            }
            const float sc = (q == 0 && a.weight) ? a.weight[j] : 1.f;
            // the item's coils in passes of CG (lanes = CG coils x tap slots)
            const int passes = MULTI ? t.passes : 1;
            if constexpr (CG == 1 && !MULTI) {
                // one coil: lane (xo, ky) takes y tap ky on every other x row from xo, so 32
                // lanes cover 16 tap slots on two rows at once
                const int ky1 = lane & 15, xo = lane >> 4;
                const float wy1 = __shfl_sync(0xffffffffu, myw, 16 + ky1);
                float2 acc1 = make_float2(0.f, 0.f);
                const float2 *rb = win + (rel0 + xo) * t.BY + rel1 + off1 + ky1;
#pragma unroll
                for (int i = 0; i < (L::WMAX + 1) / 2; ++i) {
                    if (WT == 0 && 2 * i >= W) break;
                    const int kx = 2 * i + xo;
                    const float wx = __shfl_sync(0xffffffffu, myw, kx < 16 ? kx : 15);
                    if (kx < W && ky1 < W) acc1 = __ffma2_rn(make_float2(wx, wx), rb[2 * i * t.BY], acc1);
                }
                const float wyl = ky1 < W ? wy1 : 0.f;
                float ax = wyl * acc1.x, ay = wyl * acc1.y;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    ax += __shfl_xor_sync(0xffffffffu, ax, off);
                    ay += __shfl_xor_sync(0xffffffffu, ay, off);
                }
                if (lane == 0 && it.cg0 < g.n_coil)
                    a.c[(int64_t)j * a.c_elem + (int64_t)it.cg0 * a.c_coil] = make_float2(ax * sc, ay * sc);
            } else {
                for (int ps = 0; ps < passes; ++ps) {
                    const int coil = it.cg0 + ps * CG + c;
                    float2 acc[L::KT];
#pragma unroll
                    for (int tt = 0; tt < L::KT; ++tt) acc[tt] = make_float2(0.f, 0.f);
                    const float2 *rowbase = win + (ps * CG + c) * t.CS + rel0 * t.BY + rel1 + off1;
#pragma unroll
                    for (int kx = 0; kx < L::WMAX; ++kx) {
                        if (WT == 0 && kx >= W) break;
                        float wx;
                        if constexpr (MULTI) wx = wxs[kx];
                        else wx = __shfl_sync(0xffffffffu, myw, kx);
                        const float2 wx2 = make_float2(wx, wx);
                        const float2 *row = rowbase + kx * t.BY;
#pragma unroll
                        for (int tt = 0; tt < L::KT; ++tt) {
                            const int ky = q + tt * L::NQ;
                            if (ky < W) acc[tt] = __ffma2_rn(wx2, row[ky], acc[tt]);
                        }
                    }
                    float ax = 0.f, ay = 0.f;
#pragma unroll
                    for (int tt = 0; tt < L::KT; ++tt) {
                        ax = fmaf(wy[tt], acc[tt].x, ax);
                        ay = fmaf(wy[tt], acc[tt].y, ay);
                    }
#pragma unroll
                    for (int off = CG; off < 32; off <<= 1) {
                        ax += __shfl_xor_sync(0xffffffffu, ax, off);
                        ay += __shfl_xor_sync(0xffffffffu, ay, off);
                    }
                    if (q == 0 && coil < g.n_coil)
                        a.c[(int64_t)j * a.c_elem + (int64_t)coil * a.c_coil] = make_float2(ax * sc, ay * sc);
                }
            }
        }
        __syncthreads();  // every read of this buffer (and of ring[b]) is done: refill both
        if (threadIdx.x == 0) {
            const int64_t next = item + (int64_t)S * stride;
            if (next < t.n_items) {
                ring[b] = tma_item<CG>(a, t, next);
                if (ring[b].tma) tma_issue<CG>(a, t, &map, ring[b], win, &bar[b]);
            }
        }
    }
}

}  // namespace gbn
