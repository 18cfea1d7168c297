// 3-D spread (type-1 gridding) with 8 coils per block: cubic register footprints fed by
// producer warps through an mbarrier ring.
//
// Output-stationary like k_spread3d_reg: a work item owns one output tile (or a slice of a
// dense tile's samples) and every output cell is summed by one thread, in the sample order.
// The tile (TX, TY, TZ), all multiples of 4, is cut into NWC cubes of 4 x 4 x 4 cells, one
// per consumer warp.  Lane (q, c) of a consumer warp holds coil c (8 coils) of the 4 x 4
// (y, z) cells of x plane q of its cube: 16 complex accumulators in registers.  A 12-tap
// stencil reaches a cube in ~3.75 of every 4 cells per axis on average, so ~51 % of the
// packed FMAs carry a non-zero weight, against ~36 % for the 1 x 4 x 16-cell warp rows of
// k_spread3d_reg.
//
// Staging is decoupled from the arithmetic.  The block walks a fixed sequence of (work
// item, coil group) units -- block b takes units b, b + gridDim.x, ...; the launcher gives
// one unit per block -- and numbers their 32-sample batches consecutively.  Batch t goes to
// slot t % kCubeSlots of a ring in shared memory and is filled by producer warp
// t % kCubeProducers: sample records (read by sample index), the separable
// weights of every tile plane / row / column in FP32, the 8 coil values times the optional
// density weight, and for every consumer warp the ordered list of the batch's samples whose
// stencil reaches its cube, built by ballots.  The producer waits on the slot's `empty`
// mbarrier until every consumer lane has released the slot's previous batch, and arrives on
// `full` when its writes are done.  Consumer warps walk the same sequence: wait on `full`,
// run their own list, arrive on `empty`; after a unit's last batch they write their cube
// and start the next unit from zero.  No block-wide barrier runs after the set-up: a
// consumer warp with a long list in one batch is evened out by short lists in the next
// fifteen.  (Cubes of one tile also get unequal shares of its samples over a whole unit -- a
// tile's samples cluster on one side -- which the ring cannot absorb; on the 3-D radial
// workload the cube warps' work per tile is 84 % balanced.)
//
// Every wait is bounded (kTmaWaitLimit probes of ~1 us); a wait that gives up sets
// kStatusSpreadTimeout in the plan's status word and goes on with the slot as it is, so no
// launch can hang; list lengths and entries are clamped to the batch, so such a slot is
// read in bounds.
//
// KAHAN: the instance for dense work items (kDenseFlag), with blocked Kahan summation of
// each batch's partial sums as in k_spread3d_reg.  Each instance walks the units of its own
// kind and skips the others.
#pragma once

#include "common.cuh"
#include "grid2d_kernels.cuh"
#include "grid3d_kernels.cuh"
#include "tma.cuh"

namespace gbn {

#ifndef GBN_CUBE_SLOTS
#define GBN_CUBE_SLOTS 16
#endif
// ring depth (batches), a multiple of kCubeProducers: a fast consumer warp may run up to 15
// batches ahead of the slowest (measured on the 3-D radial workload: 8 slots 11.93 ms,
// 12 slots 11.68 ms, 16 slots 11.32 ms, with 2048-sample work items)
constexpr int kCubeSlots = GBN_CUBE_SLOTS;
constexpr int kCubeProducers = 4;             // producer warps; producer p fills slots p, p + 4, ...
constexpr int kCubeBatch = 32;                // samples per batch
constexpr uint32_t kStatusSpreadTimeout = 4u; // status-word bit: a spread ring wait gave up

struct CubeLayout {
    int TX, TY, TZ;    // tile
    int CY, CZ;        // cubes along y, z (cubes along x = NWC / (CY * CZ))
    int TWP;           // floats per staged weight row: y [0, TY), z [TY, TY + TZ), x after
    size_t w_off, v_off, list_off, cnt_off, bar_off, bytes;  // per-block shared memory
};

__host__ __device__ inline CubeLayout cube_layout(const int tile[3], int nwc) {
    CubeLayout L;
    L.TX = tile[0];
    L.TY = tile[1];
    L.TZ = tile[2];
    L.CY = L.TY / 4;
    L.CZ = L.TZ / 4;
    L.TWP = reg_stride(L.TY + L.TZ + L.TX);
    L.w_off = 0;
    L.v_off = L.w_off + sizeof(float) * (size_t)kCubeSlots * kCubeBatch * L.TWP;
    L.list_off = L.v_off + sizeof(float2) * (size_t)kCubeSlots * kCubeBatch * 8;
    L.cnt_off = L.list_off + (size_t)kCubeSlots * nwc * kCubeBatch;
    L.bar_off = (L.cnt_off + sizeof(int) * (size_t)kCubeSlots * nwc + 7) & ~(size_t)7;
    L.bytes = L.bar_off + sizeof(uint64_t) * 2 * kCubeSlots;
    return L;
}

// the tile shapes this kernel takes: multiples of 4 per axis, NWC cubes of 4^3 cells
inline bool cube_tile_ok(const int tile[3], int nwc) {
    for (int d = 0; d < 3; ++d)
        if (tile[d] < 4 || tile[d] % 4 != 0) return false;
    return (tile[0] / 4) * (tile[1] / 4) * (tile[2] / 4) == nwc;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// resident blocks per SM the register allocation targets (2 fits the plain instance's
// registers without a cap)
#ifndef GBN_CUBE_MIN_BLOCKS
#define GBN_CUBE_MIN_BLOCKS 2
#endif

// loads the unit's work item; false for a unit of the other instance's kind
__device__ __forceinline__ bool cube_unit(const int4 *subs, int64_t unit, int n_cg, bool kahan, int4 &sub) {
    sub = subs[unit / n_cg];
    return ((sub.w & kDenseFlag) != 0) == kahan;
}

template <int WT, int NWC, bool KAHAN>
__global__ void __launch_bounds__((NWC + kCubeProducers) * 32, (KAHAN || NWC > 8) ? 1 : GBN_CUBE_MIN_BLOCKS)
    k_spread3d_cube(SpreadArgs a, uint32_t *status, int vec_store, int64_t n_units, int n_cg) {
    constexpr int CG = 8;
    constexpr int B = kCubeBatch;
    extern __shared__ __align__(16) unsigned char smem_cube[];
    const Geom &g = a.g;
    const CubeLayout Ly = cube_layout(g.tile, NWC);
    float *st_w = reinterpret_cast<float *>(smem_cube + Ly.w_off);          // [slot][B][TWP]
    float2 *st_v = reinterpret_cast<float2 *>(smem_cube + Ly.v_off);        // [slot][B][8]
    uint8_t *st_list = smem_cube + Ly.list_off;                             // [slot][NWC][B]
    int *st_cnt = reinterpret_cast<int *>(smem_cube + Ly.cnt_off);          // [slot][NWC]
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_cube + Ly.bar_off);  // [slot]
    uint64_t *empty = full + kCubeSlots;                                    // [slot]

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int k = 0; k < kCubeSlots; ++k) {
            mbar_init(&full[k], 32);         // the slot's producer warp, every lane
            mbar_init(&empty[k], NWC * 32);  // every consumer lane
        }
        fence_barrier_init();
    }
    __syncthreads();
    const int W = WT ? WT : g.W;

    if (warp >= NWC) {
        // ---------------------------------------------------------------- producer warp
        const int p = warp - NWC;
        const int ns = g.ns;
        int64_t t = 0;  // the block's batch counter at the start of the unit
        for (int64_t unit = blockIdx.x; unit < n_units; unit += gridDim.x) {
            int4 sub;
            if (!cube_unit(a.subs, unit, n_cg, KAHAN, sub)) continue;
            const int nb = (sub.z + B - 1) / B;
            const int cg0 = (int)(unit % n_cg) * CG;
            const int64_t stride = max(1, sub.w >> kStrideShift);  // interleaved item of a split tile
            int o[3], e[3];
            tile_coords<3>(g, sub.x % g.ntiles, o, e);
            // this producer's batches of the unit: t + k with (t + k) % kCubeProducers == p
            const int k0 = (int)((p - t % kCubeProducers + kCubeProducers) % kCubeProducers);
            for (int k = k0; k < nb; k += kCubeProducers) {
                const int64_t tb = t + k;
                const int slot = (int)(tb % kCubeSlots);
                const int n = min(B, sub.z - k * B);
                const bool ok = lane < n;
                float4 pt = make_float4(0.f, 0.f, 0.f, 0.f);
                uint32_t j = 0;
                if (ok) {
                    // the record by sample index: the 16-byte copies of the dup list would
                    // be read once per (sample, tile) pair from DRAM; the sample-order array
                    // stays in L2
                    j = a.idx[(int64_t)sub.y + (int64_t)(k * B + lane) * stride];
                    pt = a.pts_by_sample[j];
                }
                float2 v[CG];
                float sw = 1.f;
                if (ok && a.weight) sw = a.weight[j];
#pragma unroll
                for (int cc = 0; cc < CG; ++cc) {
                    v[cc] = make_float2(0.f, 0.f);
                    if (ok && cg0 + cc < g.n_coil) {
                        const float2 tv = a.c[(int64_t)j * a.c_elem + (int64_t)(cg0 + cc) * a.c_coil];
                        v[cc] = make_float2(tv.x * sw, tv.y * sw);
                    }
                }
                int r[3] = {0, 0, 0};
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
                // the slot's previous batch must be released by every consumer lane
                if (tb >= kCubeSlots &&
                    !mbar_wait_bounded(&empty[slot], (uint32_t)((tb / kCubeSlots - 1) & 1)) && lane == 0)
                    atomicOr(status, kStatusSpreadTimeout);
                float *dst = st_w + ((size_t)slot * B + lane) * Ly.TWP;
                for (int k4 = 0; k4 < Ly.TY; k4 += 4)
                    *reinterpret_cast<float4 *>(dst + k4) = make_float4(
                        tap_weight(ok, k4 - r[1], W, pt.y, ns, g.beta2[1]),
                        tap_weight(ok, k4 + 1 - r[1], W, pt.y, ns, g.beta2[1]),
                        tap_weight(ok, k4 + 2 - r[1], W, pt.y, ns, g.beta2[1]),
                        tap_weight(ok, k4 + 3 - r[1], W, pt.y, ns, g.beta2[1]));
                for (int k4 = 0; k4 < Ly.TZ; k4 += 4)
                    *reinterpret_cast<float4 *>(dst + Ly.TY + k4) = make_float4(
                        tap_weight(ok, k4 - r[2], W, pt.z, ns, g.beta2[2]),
                        tap_weight(ok, k4 + 1 - r[2], W, pt.z, ns, g.beta2[2]),
                        tap_weight(ok, k4 + 2 - r[2], W, pt.z, ns, g.beta2[2]),
                        tap_weight(ok, k4 + 3 - r[2], W, pt.z, ns, g.beta2[2]));
                for (int k4 = 0; k4 < Ly.TX; k4 += 4)
                    *reinterpret_cast<float4 *>(dst + Ly.TY + Ly.TZ + k4) = make_float4(
                        tap_weight(ok, k4 - r[0], W, pt.x, ns, g.beta2[0]),
                        tap_weight(ok, k4 + 1 - r[0], W, pt.x, ns, g.beta2[0]),
                        tap_weight(ok, k4 + 2 - r[0], W, pt.x, ns, g.beta2[0]),
                        tap_weight(ok, k4 + 3 - r[0], W, pt.x, ns, g.beta2[0]));
                float4 *vd = reinterpret_cast<float4 *>(st_v + ((size_t)slot * B + lane) * CG);
#pragma unroll
                for (int cc = 0; cc < CG; cc += 2)
                    vd[cc / 2] = make_float4(v[cc].x, v[cc].y, v[cc + 1].x, v[cc + 1].y);
                // per consumer warp: the samples whose stencil reaches its cube, in order
                uint8_t *lst = st_list + (size_t)slot * NWC * B;
                for (int w = 0; w < NWC; ++w) {
                    const int cx = 4 * (w / (Ly.CY * Ly.CZ)), cy = 4 * ((w / Ly.CZ) % Ly.CY), cz = 4 * (w % Ly.CZ);
                    const bool hit = ok && r[0] < cx + 4 && r[0] + W > cx && r[1] < cy + 4 && r[1] + W > cy &&
                                     r[2] < cz + 4 && r[2] + W > cz;
                    const unsigned m = __ballot_sync(0xffffffffu, hit);
                    if (hit) lst[w * B + __popc(m & lanemask_lt(lane))] = (uint8_t)lane;
                    if (lane == 0) st_cnt[slot * NWC + w] = __popc(m);
                }
                mbar_arrive(&full[slot]);
            }
            t += nb;
        }
        return;
    }

    // -------------------------------------------------------------------- consumer warp
    const int c = lane & 7, q = lane >> 3;
    const int cx = 4 * (warp / (Ly.CY * Ly.CZ)), cy = 4 * ((warp / Ly.CZ) % Ly.CY), cz = 4 * (warp % Ly.CZ);
    const int wxo = Ly.TY + Ly.TZ + cx + q;  // this lane's x-plane weight in a staged row
    int64_t t = 0;
    for (int64_t unit = blockIdx.x; unit < n_units; unit += gridDim.x) {
        int4 sub;
        if (!cube_unit(a.subs, unit, n_cg, KAHAN, sub)) continue;
        const int nb = (sub.z + B - 1) / B;
        const int cg0 = (int)(unit % n_cg) * CG;
        float2 acc[4][4];
        float2 tot[KAHAN ? 4 : 1][KAHAN ? 4 : 1], cmp[KAHAN ? 4 : 1][KAHAN ? 4 : 1];
#pragma unroll
        for (int rr = 0; rr < 4; ++rr)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[rr][k] = make_float2(0.f, 0.f);
        if constexpr (KAHAN) {
#pragma unroll
            for (int rr = 0; rr < 4; ++rr)
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    tot[rr][k] = make_float2(0.f, 0.f);
                    cmp[rr][k] = make_float2(0.f, 0.f);
                }
        }
        for (int k = 0; k < nb; ++k, ++t) {
            const int slot = (int)(t % kCubeSlots);
            if (!mbar_wait_bounded(&full[slot], (uint32_t)((t / kCubeSlots) & 1)) && lane == 0)
                atomicOr(status, kStatusSpreadTimeout);
            const float *wbase = st_w + (size_t)slot * B * Ly.TWP;
            const float2 *vbase = st_v + (size_t)slot * B * CG;
            const uint8_t *lst = st_list + ((size_t)slot * NWC + warp) * B;
            const int cnt = min(st_cnt[slot * NWC + warp], B);
            for (int i = 0; i < cnt; ++i) {
                const int s = lst[i] & (B - 1);
                const float *w = wbase + s * Ly.TWP;
                const float2 v0 = vbase[s * CG + c];
                const float wx = w[wxo];
                const float4 wy = *reinterpret_cast<const float4 *>(w + cy);
                const float4 wz = *reinterpret_cast<const float4 *>(w + Ly.TY + cz);
                const float2 v = make_float2(wx * v0.x, wx * v0.y);
                const float2 u[4] = {make_float2(wz.x * v.x, wz.x * v.y), make_float2(wz.y * v.x, wz.y * v.y),
                                     make_float2(wz.z * v.x, wz.z * v.y), make_float2(wz.w * v.x, wz.w * v.y)};
                const float wyr[4] = {wy.x, wy.y, wy.z, wy.w};
#pragma unroll
                for (int rr = 0; rr < 4; ++rr) {
                    const float2 wy2 = make_float2(wyr[rr], wyr[rr]);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) acc[rr][kk] = __ffma2_rn(wy2, u[kk], acc[rr][kk]);
                }
            }
            mbar_arrive(&empty[slot]);
            if constexpr (KAHAN) {
#pragma unroll
                for (int rr = 0; rr < 4; ++rr)
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        kahan_add(tot[rr][kk], cmp[rr][kk], acc[rr][kk]);
                        acc[rr][kk] = make_float2(0.f, 0.f);
                    }
            }
        }
        if constexpr (KAHAN) {
#pragma unroll
            for (int rr = 0; rr < 4; ++rr)
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    acc[rr][k] = make_float2(tot[rr][k].x - cmp[rr][k].x, tot[rr][k].y - cmp[rr][k].y);
        }

        // write this unit's cube (each cell has one owner, so no other warp waits for it)
        int o[3], e[3];
        tile_coords<3>(g, sub.x % g.ntiles, o, e);
        const int grp = sub.x / g.ntiles;
        const int lx = cx + q;
        if (cg0 + c >= g.n_coil || lx >= e[0]) continue;
        const bool split = (sub.w & kSplitFlag) != 0;
        float2 *dstc = a.grid + ((int64_t)grp * g.n_coil + cg0 + c) * g.G + (int64_t)(o[0] + lx) * g.nf[1] * g.nf[2];
        const bool zfull = vec_store && cz + 4 <= e[2];
#pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
            const int ly = cy + rr;
            if (ly >= e[1]) break;
            float2 *row = dstc + (int64_t)(o[1] + ly) * g.nf[2] + (o[2] + cz);
            if (split) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (cz + k >= e[2]) break;
                    atomicAdd(&row[k].x, acc[rr][k].x);
                    atomicAdd(&row[k].y, acc[rr][k].y);
                }
            } else if (zfull) {
                // cells (z, z+1) as one 16-byte store: o[2] + cz is a multiple of 4 and, with
                // vec_store (grid 16-byte aligned, nf[2] even), every row starts 16-byte aligned
                float4 *r4 = reinterpret_cast<float4 *>(row);
                r4[0] = make_float4(acc[rr][0].x, acc[rr][0].y, acc[rr][1].x, acc[rr][1].y);
                r4[1] = make_float4(acc[rr][2].x, acc[rr][2].y, acc[rr][3].x, acc[rr][3].y);
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (cz + k >= e[2]) break;
                    row[k] = acc[rr][k];
                }
            }
        }
    }
}

}  // namespace gbn
