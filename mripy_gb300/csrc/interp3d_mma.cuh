// 3-D interp (type-2 gridding) of 8 coils on the tensor cores.
//
// The forward gridding of sample s is out[s, c] = sum_{x,y,z} wx_s[x] wy_s[y] wz_s[z] G[x,y,z,c].
// Restricted to one tile of the spread's 4 x 8 x 16 tiling, with the separable weights
// split the same way as in k_spread_mma, its (y, z) part is a GEMM with the samples as M:
//     T[s, (x, c, re/im)] = sum_{(y,z)} A[s, (y, z)] * B[(x, c, re/im), (y, z)]
//     A[s, (y, z)] = wy_s[y] wz_s[z]          (M = 128 samples, K = 8 x 16 = 128 cells)
//     B = the tile's grid values               (N = 4 x 8 x 2 = 64)
// and the x part is a per-sample contraction partial[s, c] = sum_x wx_s[x] T[s, (x, c)].  A
// sample's result is the sum of its partials over the ~15 tiles its stencil reaches (the
// spread's (sample, tile) work lists), added into the zeroed output with float atomics.
//
// One (work item, coil group) unit per block, 9 warps; a block whose work item is empty
// leaves at once.  At the start the builders issue their first samples' index loads, then
// all threads load the tile's 8 coils x 512 cells (two z cells per 16-byte load where the
// grid's alignment allows), split them into TF32 hi + lo parts and write B into shared
// memory (K-major, 128-byte swizzle, four 32-column K atoms of two y rows each). Then per
// batch of 128 of the unit's samples:
// * 8 builder warps: warp (q, h) takes samples 32 q .. 32 q + 31 of the batch, one per lane
//   (TMEM lane = sample), reads its record, computes its plane weights (ex2.approx) and writes
//   A in four chunks of 32 columns (y rows 2 c and 2 c + 1; warp h writes row 2 c + h) into
//   two TMEM chunk buffers, hi and lo parts, arriving on the buffer's `ops` mbarrier; after
//   the batch it finishes the previous batch: reads its 32 columns of T (coils 4 h .. 4 h + 3,
//   every x) from TMEM, contracts them with wx and adds them to the output.
// * 1 MMA warp: allocates 256 TMEM columns (A chunks 0..127, two accumulators T 128..255) and
//   issues per chunk 4 K steps x 3 MMAs (hi * hi, hi * lo, lo * hi) into the batch's T,
//   committing each chunk to its buffer's `done` mbarrier and the batch to `tfull`.
// Every wait is bounded (kTmaWaitLimit probes); one that gives up sets kStatusSpreadTimeout
// in the plan's status word and goes on.
#pragma once

#include "common.cuh"
#include "grid_kernels.cuh"
#include "spread3d_mma.cuh"
#include "tc.cuh"

namespace gbn {

constexpr int kImBatch = 128;                  // samples per batch: TMEM lanes
constexpr int kImBuilders = 8;
constexpr int kImWarp = kImBuilders;           // the MMA warp's index
constexpr int kImThreads = 32 * (kImBuilders + 1);
constexpr uint32_t kImTmemCols = 256;          // A chunks (hi 32 + lo 32) x 2: 0..127; T x 2: 128..255
constexpr uint32_t kImColT = 128;
constexpr uint32_t kImBAtom = kMmaN * 128;     // one 32-column K atom of B: 64 rows x 128 B
constexpr uint32_t kImBOp = 4 * kImBAtom;      // B hi (or lo): 32 KB
constexpr uint32_t kImBarOff = 2 * kImBOp;
constexpr uint32_t kImBars = 8;                // ops[2], done[2], tfull[2], tempty[2]
// above a third of the SM's 228 KB: at most two blocks (2 x 256 TMEM columns) per SM
constexpr size_t kImSmemBytes = 78 * 1024;
static_assert(kImBarOff + 8 * kImBars + 16 + 1024 <= kImSmemBytes, "interp smem layout");
static_assert(kImSmemBytes > 228 * 1024 / 3, "two blocks per SM at most");

// byte offset of B element (row n, K index k = y * 16 + z): K atom k / 32, 128-byte swizzle
__device__ __forceinline__ uint32_t im_b_offset(int n, int k) {
    return (uint32_t)(k >> 5) * kImBAtom + sw128_offset(n, k & 31);
}

template <int WT>
__global__ void __launch_bounds__(kImThreads, 2) k_interp3d_mma(MmaInterpArgs a, uint32_t *status, int n_cg,
                                                                 int vec_atomic) {
    constexpr int B = kImBatch;
    constexpr int CG = 8;
    extern __shared__ unsigned char smem_im_raw[];
    unsigned char *sm = smem_im_raw + ((1024u - (smem_addr(smem_im_raw) & 1023u)) & 1023u);
    unsigned char *bh = sm, *bl = sm + kImBOp;
    uint64_t *ops = reinterpret_cast<uint64_t *>(sm + kImBarOff);
    uint64_t *done = ops + 2;
    uint64_t *tfull = done + 2;
    uint64_t *tempty = tfull + 2;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(tempty + 2);

    const Geom &g = a.g;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = WT ? WT : g.W;
    const int64_t unit = blockIdx.x;
    const int4 sub = a.subs[unit / n_cg];
    const int cg0 = (int)(unit % n_cg) * CG;
    const int grp = sub.x / g.ntiles;
    int o[3], e[3];
    tile_coords<3>(g, sub.x % g.ntiles, o, e);
    const int nb = (sub.z + kImBatch - 1) / kImBatch;
    if (nb == 0) return;  // an empty work item: no sample to add to (the launcher zeroed them)

    if (warp == kImWarp) {
        tmem_alloc(tslot, kImTmemCols);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int b = 0; b < 2; ++b) {
            mbar_init(&ops[b], kImBuilders * 32);
            mbar_init(&done[b], 1);
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kImBuilders * 32);
        }
        fence_barrier_init();
    }
    // the builders' first sample indices, read before the tile so that their latency
    // overlaps its loads (each builder lane: sample 32 q + lane of the first batch)
    const int64_t stride = max(1, sub.w >> kStrideShift);  // interleaved item of a split tile
    uint32_t jn = 0;
    bool okn = warp != kImWarp && 32 * (warp & 3) + lane < sub.z;
    if (okn) jn = a.idx[(int64_t)sub.y + (int64_t)(32 * (warp & 3) + lane) * stride];
    // B: the tile's cells (x, y, z) of the 8 coils; cells past the grid edge and padded
    // coils are 0.  z fastest across threads: 128-byte runs of each (coil, x, y) row.
    // Loads are issued 8 at a time before any is used, so a thread waits for one memory
    // latency per 8 cells rather than per cell.
    constexpr int kCells = CG * kMmaTX * kMmaTY * kMmaTZ;
    const float2 *base = a.grid + (int64_t)grp * g.n_coil * g.G;
    if (vec_atomic & 2) {
        // pairs of z cells, one 16-byte load each: a partial tile's z extent is even too
        static_assert(kCells / 2 <= 8 * kImThreads, "one round of loads");
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = threadIdx.x + u * kImThreads;  // pair index
            const int z = 2 * (i & 7), y = (i >> 3) & 7, x = (i >> 6) & 3, c = i >> 8;
            v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (i < kCells / 2 && cg0 + c < g.n_coil && x < e[0] && y < e[1] && z < e[2])
                v[u] = *reinterpret_cast<const float4 *>(
                    base + (int64_t)(cg0 + c) * g.G + ((int64_t)(o[0] + x) * g.nf[1] + (o[1] + y)) * g.nf[2] + (o[2] + z));
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = threadIdx.x + u * kImThreads;
            if (i >= kCells / 2) break;
            const int z = 2 * (i & 7), y = (i >> 3) & 7, x = (i >> 6) & 3, c = i >> 8;
#pragma unroll
            for (int hz = 0; hz < 2; ++hz) {
                float2 h, l;
                tf32_split2(hz ? make_float2(v[u].z, v[u].w) : make_float2(v[u].x, v[u].y), make_float2(1.f, 1.f), h, l);
                const int n = x * 16 + c * 2, k = y * 16 + z + hz;
                const uint32_t ore = im_b_offset(n, k), oim = im_b_offset(n + 1, k);
                *reinterpret_cast<float *>(bh + ore) = h.x;
                *reinterpret_cast<float *>(bl + ore) = l.x;
                *reinterpret_cast<float *>(bh + oim) = h.y;
                *reinterpret_cast<float *>(bl + oim) = l.y;
            }
        }
    } else
    for (int r0 = threadIdx.x; r0 < kCells; r0 += 8 * kImThreads) {
        float2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = r0 + u * kImThreads;
            const int z = i & 15, y = (i >> 4) & 7, x = (i >> 7) & 3, c = i >> 9;
            v[u] = make_float2(0.f, 0.f);
            if (i < kCells && cg0 + c < g.n_coil && x < e[0] && y < e[1] && z < e[2])
                v[u] = base[(int64_t)(cg0 + c) * g.G + ((int64_t)(o[0] + x) * g.nf[1] + (o[1] + y)) * g.nf[2] +
                            (o[2] + z)];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = r0 + u * kImThreads;
            if (i >= kCells) break;
            const int z = i & 15, y = (i >> 4) & 7, x = (i >> 7) & 3, c = i >> 9;
            float2 h, l;
            tf32_split2(v[u], make_float2(1.f, 1.f), h, l);
            const int n = x * 16 + c * 2, k = y * 16 + z;
            const uint32_t ore = im_b_offset(n, k), oim = im_b_offset(n + 1, k);
            *reinterpret_cast<float *>(bh + ore) = h.x;
            *reinterpret_cast<float *>(bl + ore) = l.x;
            *reinterpret_cast<float *>(bh + oim) = h.y;
            *reinterpret_cast<float *>(bl + oim) = l.y;
        }
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;

    if (warp == kImWarp) {
        // ---------------------------------------------------------------- MMA warp
        if (lane == 0) {
            constexpr uint32_t idesc = tc_idesc_tf32(kImBatch, kMmaN);
            // descriptors of B's first K step; a K step's offset adds (bytes / 16) to the
            // address field (shared addresses stay far below its 14-bit range)
            const uint64_t dbh = tc_desc_sw128(smem_addr(bh)), dbl = tc_desc_sw128(smem_addr(bl));
            for (int b = 0; b < nb; ++b) {
                const int tb = b & 1;
                // T[tb] was read out by the builders (batch b - 2)
                if (b >= 2 && !mbar_wait_bounded(&tempty[tb], (uint32_t)(((b >> 1) - 1) & 1)))
                    atomicOr(status, kStatusSpreadTimeout);
                const uint32_t d = tbase + kImColT + 64u * tb;
#pragma unroll
                for (int ch = 0; ch < 4; ++ch) {
                    const int gch = 4 * b + ch, buf = gch & 1;
                    if (!mbar_wait_bounded(&ops[buf], (uint32_t)((gch >> 1) & 1))) atomicOr(status, kStatusSpreadTimeout);
                    tc_fence_after();
                    const uint32_t ah = tbase + 64u * buf, al = ah + 32u;
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks) {
                        const uint64_t kb = ((uint64_t)ch * kImBAtom + 32u * ks) >> 4;
                        tc_mma_tf32_ts(d, ah + 8u * ks, dbh + kb, idesc, (ch | ks) != 0);
                        tc_mma_tf32_ts(d, ah + 8u * ks, dbl + kb, idesc, 1u);
                        tc_mma_tf32_ts(d, al + 8u * ks, dbh + kb, idesc, 1u);
                    }
                    tc_commit(&done[buf]);
                }
                tc_commit(&tfull[tb]);
            }
        }
        __syncwarp();
    } else {
        // ---------------------------------------------------------------- builder warp
        const int q = warp & 3, h = warp >> 2;
        const uint32_t tl = tmem_lane_base(tbase, q);
        const int ns = g.ns;
        // the previous batch's sample for the deferred epilogue
        float wxp[4] = {0.f, 0.f, 0.f, 0.f};
        uint32_t jp = 0;
        bool okp = false;
        // records are read one batch ahead: the next batch's entry early in the batch, its
        // sample record half way through, so neither load is waited for where it is used
        float4 ptn = make_float4(0.f, 0.f, 0.f, 0.f);
        if (okn) ptn = a.pts_by_sample[jn];
        for (int b = 0; b <= nb; ++b) {
            float wx[4] = {0.f, 0.f, 0.f, 0.f};
            uint32_t j = 0;
            bool ok = false;
            if (b < nb) {
                j = jn;
                ok = okn;
                const float4 pt = ptn;
                {
                    const int i = (b + 1) * B + 32 * q + lane;
                    okn = i < sub.z;
                    if (okn) jn = a.idx[(int64_t)sub.y + (int64_t)i * stride];
                }
                // per dimension the first tap's tile plane r and the distance of plane 0
                int r[3] = {-(1 << 20), -(1 << 20), -(1 << 20)};
                if (ok) {
                    int c0[3];
                    unpack_cells(3, __float_as_uint(pt.w), c0[0], c0[1], c0[2]);
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        int rr = c0[d] - o[d];
                        rr += rr < 0 ? g.nf[d] : 0;
                        rr -= rr > g.nf[d] - W ? g.nf[d] : 0;
                        r[d] = rr;
                    }
                }
                const float d0x = pt.x + (float)(ns - 1 + r[0]);
                const float d0y = pt.y + (float)(ns - 1 + r[1]);
                const float d0z = pt.z + (float)(ns - 1 + r[2]);
#pragma unroll
                for (int t = 0; t < kMmaTX; ++t) {
                    const float d = d0x - (float)t;
                    const float wv = ex2_approx(-g.beta2[0] * d * d);
                    wx[t] = (unsigned)(t - r[0]) < (unsigned)W ? wv : 0.f;
                }
                float wz[kMmaTZ];
#pragma unroll
                for (int t = 0; t < kMmaTZ; ++t) {
                    const float d = d0z - (float)t;
                    const float wv = ex2_approx(-g.beta2[2] * d * d);
                    wz[t] = (unsigned)(t - r[2]) < (unsigned)W ? wv : 0.f;
                }
#pragma unroll
                for (int ch = 0; ch < 4; ++ch) {
                    const int gch = 4 * b + ch, buf = gch & 1;
                    // the MMAs of chunk gch - 2 (same buffer) have completed
                    if (gch >= 2 && !mbar_wait_bounded(&done[buf], (uint32_t)(((gch >> 1) - 1) & 1)) && lane == 0)
                        atomicOr(status, kStatusSpreadTimeout);
                    if (ch == 1 && okn) ptn = a.pts_by_sample[jn];
                    const int y = 2 * ch + h;
                    const float dy = d0y - (float)y;
                    const float wyv = ex2_approx(-g.beta2[1] * dy * dy);
                    const float wy = (unsigned)(y - r[1]) < (unsigned)W ? wyv : 0.f;
                    float hi[16], lo[16];
#pragma unroll
                    for (int t = 0; t < kMmaTZ; t += 2) {
                        float2 hh, ll;
                        tf32_split2(make_float2(wy, wy), make_float2(wz[t], wz[t + 1]), hh, ll);
                        hi[t] = hh.x;
                        hi[t + 1] = hh.y;
                        lo[t] = ll.x;
                        lo[t + 1] = ll.y;
                    }
                    tmem_st_x16(tl + 64u * buf + 16u * h, hi);
                    tmem_st_x16(tl + 64u * buf + 32u + 16u * h, lo);
                    tmem_wait_st();
                    tc_fence_before();
                    mbar_arrive(&ops[buf]);
                }
            }
            if (b >= 1) {
                // epilogue of batch b - 1: coils 4 h .. 4 h + 3, every x plane
                const int pb = b - 1, tb = pb & 1;
                if (!mbar_wait_bounded(&tfull[tb], (uint32_t)((pb >> 1) & 1)) && lane == 0)
                    atomicOr(status, kStatusSpreadTimeout);
                tc_fence_after();
                float tv[4][8];
#pragma unroll
                for (int x = 0; x < 4; ++x) {
                    float t8[8];
                    tmem_ld_x8(tl + kImColT + 64u * tb + 16u * x + 8u * h, t8);
#pragma unroll
                    for (int i = 0; i < 8; ++i) tv[x][i] = t8[i];
                }
                tmem_wait_ld();
                tc_fence_before();
                mbar_arrive(&tempty[tb]);
                if (okp) {
                    const float sc = a.weight ? a.weight[jp] : 1.f;
                    float pr[8];
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) {
                        float re = 0.f, im = 0.f;
#pragma unroll
                        for (int x = 0; x < 4; ++x) {
                            re = fmaf(wxp[x], tv[x][2 * cc], re);
                            im = fmaf(wxp[x], tv[x][2 * cc + 1], im);
                        }
                        pr[2 * cc] = re * sc;
                        pr[2 * cc + 1] = im * sc;
                    }
                    const int coil0 = cg0 + 4 * h;
                    float2 *dst = a.c + (int64_t)jp * a.c_elem + (int64_t)coil0 * a.c_coil;
                    if ((vec_atomic & 1) && coil0 + 4 <= g.n_coil) {
                        // coils adjacent and 16-byte aligned: two coils per atomic
                        atomicAdd(reinterpret_cast<float4 *>(dst), make_float4(pr[0], pr[1], pr[2], pr[3]));
                        atomicAdd(reinterpret_cast<float4 *>(dst + 2), make_float4(pr[4], pr[5], pr[6], pr[7]));
                    } else {
#pragma unroll
                        for (int cc = 0; cc < 4; ++cc) {
                            if (coil0 + cc >= g.n_coil) break;
                            atomicAdd(dst + (int64_t)cc * a.c_coil, make_float2(pr[2 * cc], pr[2 * cc + 1]));
                        }
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < 4; ++t) wxp[t] = wx[t];
            jp = j;
            okp = ok;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kImWarp) tmem_dealloc(tbase, kImTmemCols);
}

}  // namespace gbn
