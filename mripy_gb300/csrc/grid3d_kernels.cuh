// 3-D gridding kernels with warp-level accumulation (the same design as the 2-D kernels,
// with z as the lane direction).
//
// Lane mapping: lane = c + CG*q, coil c in [0, CG), z-tap slot q in [0, NQ); slot q handles
// kz = q, q+NQ, ... (KT taps).  Shared-memory layout [x][y][z][coil]: for one (x, y) row a
// warp touches NQ*KT consecutive z cells of CG consecutive coils, one contiguous run.
//
// Interp: one warp per sample over the staged window of its home bin (tile + W - 1 cells per
// dimension, periodic wrap).  Lanes 0..15 evaluate wx, lanes 16..31 wy (one exp2 each), every
// lane evaluates the wz of its own taps; each lane then sums its W*W*KT taps for its coil
// and a shuffle reduction over the slots yields the coil value.
//
// Spread: output-stationary tile [TX][TY][TZ][CG]; warp w owns the x-planes
// [w*P, (w+1)*P).  Samples are staged in batches (weights, weighted coil values, signed local
// first-tap cells); every warp walks the batch and applies the taps in its own planes with
// plain load-add-store (no atomics, fixed order).  Signed local coordinates are exact when
// nf >= tile + W in every dimension; smaller grids use the generic kernels.
#pragma once

#include "grid2d_kernels.cuh"
#include "grid_kernels.cuh"
#include "tma.cuh"

namespace gbn {

inline bool grid3d_applies(const Geom &g) {
    return g.dim == 3 && g.W <= 16 && g.nf[0] >= g.tile[0] + g.W && g.nf[1] >= g.tile[1] + g.W &&
           g.nf[2] >= g.tile[2] + g.W;
}

// --------------------------------------------------------------------------------- interp
template <int WT, int CG>
__global__ void __launch_bounds__(256) k_interp3d(InterpArgs a) {
    using L = Lanes2D<WT, CG>;
    extern __shared__ float4 smem_i3[];
    float2 *win = reinterpret_cast<float2 *>(smem_i3);  // [WX][WY][WZ][CG]
    const Geom &g = a.g;
    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    int o[3], e[3];
    tile_coords<3>(g, sub.x % g.ntiles, o, e);
    const int W = WT ? WT : g.W;
    const int ns = g.ns;
    const int WX = g.tile[0] + W - 1, WY = g.tile[1] + W - 1, WZ = g.tile[2] + W - 1;
    const int nf0 = g.nf[0], nf1 = g.nf[1], nf2 = g.nf[2];

    {
        const int ws0 = o[0] - (ns - 1), ws1 = o[1] - (ns - 1), ws2 = o[2] - (ns - 1);
        const float2 *base = a.grid + ((int64_t)grp * g.n_coil + cg0) * g.G;
        // coil fastest across threads: consecutive shared-memory words, CG runs of
        // consecutive z cells per warp load
        const int nitem = WX * WY * WZ * CG;
        const float rWZ = 1.f / (float)WZ, rWY = 1.f / (float)WY;
        for (int i = threadIdx.x; i < nitem; i += blockDim.x) {
            const int c = i % CG, cell = i / CG;  // CG is a power of two
            const int xy = div_small(cell, rWZ), wz = cell - xy * WZ;
            const int wx = div_small(xy, rWY), wy = xy - wx * WY;
            const int gx = wrap_fast(ws0 + wx, nf0), gy = wrap_fast(ws1 + wy, nf1), gz = wrap_fast(ws2 + wz, nf2);
            win[i] = (cg0 + c < g.n_coil) ? base[(int64_t)c * g.G + ((int64_t)gx * nf1 + gy) * nf2 + gz]
                                          : make_float2(0.f, 0.f);
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int c = lane % CG, q = lane / CG;
    const int kk = lane & 15;
    const float beta = lane < 16 ? g.beta2[0] : g.beta2[1];
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
        int c0[3];
        unpack_cells(3, __float_as_uint(p.w), c0[0], c0[1], c0[2]);
        int rel[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int cc = c0[d] + ns - 1;
            cc -= cc >= g.nf[d] ? g.nf[d] : 0;
            rel[d] = cc - o[d];
        }
        float myw = 0.f;
        if (kk < W) {
            const float d = (lane < 16 ? p.x : p.y) + (float)(ns - 1 - kk);
            myw = exp2f(-beta * d * d);
        }
        float2 acc = make_float2(0.f, 0.f);
        if constexpr (CG == 1) {
            // one coil: lane (yo, kz) takes z tap kz on every other y row from yo, so 32
            // lanes cover 16 tap slots on two rows at once; each lane's y weights come from
            // the lanes 16.. that evaluated them
            constexpr int HW = (L::WMAX + 1) / 2;
            const int kz = lane & 15, yo = lane >> 4;
            float wyl[HW];
#pragma unroll
            for (int i = 0; i < HW; ++i) wyl[i] = __shfl_sync(0xffffffffu, myw, 16 + min(2 * i + yo, 15));
            const float dz = p.z + (float)(ns - 1 - kz);
            const float wz1 = kz < W ? exp2f(-g.beta2[2] * dz * dz) : 0.f;
            float2 at1 = make_float2(0.f, 0.f);
            const float2 *base1 = win + (((size_t)rel[0] * WY + rel[1] + yo) * WZ + rel[2]) + kz;
#pragma unroll 1
            for (int kx = 0; kx < W; ++kx) {
                const float wx = __shfl_sync(0xffffffffu, myw, kx);
                const float2 *plane = base1 + (size_t)kx * WY * WZ;
#pragma unroll
                for (int i = 0; i < HW; ++i) {
                    if (WT == 0 && 2 * i >= W) break;
                    if (2 * i + yo < W && kz < W) {
                        const float wxy = wx * wyl[i];
                        at1 = __ffma2_rn(make_float2(wxy, wxy), plane[(size_t)2 * i * WZ], at1);
                    }
                }
            }
            acc = make_float2(wz1 * at1.x, wz1 * at1.y);
        } else {
            float wy[L::WMAX];
#pragma unroll
            for (int k = 0; k < L::WMAX; ++k) wy[k] = __shfl_sync(0xffffffffu, myw, 16 + k);
            float wz[L::KT];
#pragma unroll
            for (int t = 0; t < L::KT; ++t) {
                const int kz = q + t * L::NQ;
                const float d = p.z + (float)(ns - 1 - kz);
                wz[t] = kz < W ? exp2f(-g.beta2[2] * d * d) : 0.f;
            }
            // a lane's z taps are fixed: sum wx wy * G per tap slot, apply wz once at the end
            float2 at[L::KT];
#pragma unroll
            for (int t = 0; t < L::KT; ++t) at[t] = make_float2(0.f, 0.f);
            const float2 *base = win + (((size_t)rel[0] * WY + rel[1]) * WZ + rel[2]) * CG + c;
#pragma unroll 1
            for (int kx = 0; kx < W; ++kx) {
                const float wx = __shfl_sync(0xffffffffu, myw, kx);
                const float2 *plane = base + (size_t)kx * WY * WZ * CG;
#pragma unroll
                for (int ky = 0; ky < L::WMAX; ++ky) {
                    if (WT == 0 && ky >= W) break;
                    const float wxy = wx * wy[ky];
                    const float2 wxy2 = make_float2(wxy, wxy);
                    const float2 *row = plane + (size_t)ky * WZ * CG;
#pragma unroll
                    for (int t = 0; t < L::KT; ++t) {
                        const int kz = q + t * L::NQ;
                        if (kz < W) at[t] = __ffma2_rn(wxy2, row[kz * CG], at[t]);
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < L::KT; ++t) {
                acc.x = fmaf(wz[t], at[t].x, acc.x);
                acc.y = fmaf(wz[t], at[t].y, acc.y);
            }
        }
#pragma unroll
        for (int off = CG; off < 32; off <<= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, off);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, off);
        }
        if (q == 0 && cg0 + c < g.n_coil) {
            const float sc = a.weight ? a.weight[j] : 1.f;
            a.c[(int64_t)j * a.c_elem + (int64_t)(cg0 + c) * a.c_coil] = make_float2(acc.x * sc, acc.y * sc);
        }
    }
}

// ------------------------------------------------------------------ interp, plane streaming
// For 4 or 8 coils per block.  A bin's (TX+W-1) x (TY+W-1) x (TZ+W-1) window does not fit in
// shared memory at 8 coils (439 KB for 8^3 bins), so it is streamed one x plane at a time:
// two plane buffers, the next plane copied while the current one is used -- by one tensor
// copy (cp.async.bulk.tensor.4d, completing on an mbarrier; the copy writes shared memory
// outside the load/store pipe the sample loop is bound by) when the window lies inside the
// grid in y and z, else by the threads with cp.async (periodic wrap at the grid edge).  Up
// to kPlaneSamples samples of the bin are processed together; their weights
// (16 slots per dimension), home-relative first taps and per-coil accumulators live in
// shared memory.  For each plane every warp walks its samples (sample s belongs to warp
// s mod warps); a sample whose x stencil covers the plane adds wx * sum_y wy sum_z wz G over
// the plane's W x W taps: lanes = (coil, z slot) as in k_interp3d, per-slot sums applied
// with wz once, a shuffle reduction over the slots, and one lane per coil adding the result
// to the sample's accumulator (no other warp touches it).  A plane is stored coil-major,
// [coil][y][z] in the copy box's layout (plane_box), so the threads' copies run along z
// (contiguous in the grid) and the lanes' reads stay conflict-free.  (With coil-fastest
// planes each 8-byte copy of a warp came from a different coil volume and cost its own
// shared-memory wavefront: 40 % of the shared pipe of the c4 launch went to staging.)
constexpr int kPlaneMaxElems = 4096;  // plane elements (coil stride x coils) the kernel accepts

// 8-byte asynchronous copy global -> shared (cp.async); src_bytes 0 writes zeros
__device__ __forceinline__ void cp_async8(void *dst, const void *src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Staged plane [coil][y][z]: BY rows of BZ cells per coil, coil stride BY * BZ.  This is
// the box of the plane's tensor copy (z innermost): BZ is even and covers the window's z
// extent plus one cell, because the copy starts on an even z cell (16-byte boundary); BY
// covers the y extent.  BY * BZ is chosen so that a half-warp's 8-byte reads (CG coils x
// 16/CG consecutive z cells) fall on 32 distinct banks: 8 coils -> 2 mod 4 (coil c starts
// 4c words apart, mod 32), 4 coils -> 4 mod 8 (8c words apart).  The threads' copies (windows
// that wrap at the periodic grid edge) use the same layout.
struct PlaneBox {
    int BY, BZ;
};
__host__ __device__ inline PlaneBox plane_box(const Geom &g, int cg) {
    const int WY = g.tile[1] + g.W - 1, WZ = g.tile[2] + g.W - 1;
    const int m = cg == 8 ? 4 : 8, r = cg == 8 ? 2 : 4;
    for (int bz = (WZ + 2) & ~1; bz < WZ + 18; bz += 2)
        for (int by = WY; by < WY + 4; ++by)
            if ((by * bz) % m == r) return PlaneBox{by, bz};
    return PlaneBox{0, 0};
}
// float2 per plane buffer, rounded to 128 bytes (tensor-copy destinations)
__host__ __device__ inline int plane_elems(const PlaneBox &b, int cg) { return (b.BY * b.BZ * cg + 15) & ~15; }

// the threads' copy of plane gx (periodic y/z indices) into dst: consecutive threads take
// consecutive z cells of one coil, so a warp's sources are contiguous runs in the grid and
// its shared-memory writes consecutive words.  The caller waits (cp_async_wait_all) and
// synchronises before reading it.
template <int CG>
__device__ __forceinline__ void plane_copy(float2 *dst, const float2 *__restrict__ base, const Geom &g, int cg0,
                                           int gx, int ws1, int ws2, int WZ, int cells, int BZ, int CSP, float rWZ,
                                           float rcells) {
    const float2 *pb = base + (int64_t)gx * g.nf[1] * g.nf[2];
    for (int el = threadIdx.x; el < CG * cells; el += blockDim.x) {
        const int cc = div_small(el, rcells), cell = el - cc * cells;
        const int wy = div_small(cell, rWZ), wz = cell - wy * WZ;
        const int gy = wrap_fast(ws1 + wy, g.nf[1]), gz = wrap_fast(ws2 + wz, g.nf[2]);
        const bool ok = cg0 + cc < g.n_coil;
        const float2 *src = ok ? pb + (int64_t)cc * g.G + (int64_t)gy * g.nf[2] + gz : pb;
        cp_async8(dst + cc * CSP + wy * BZ + wz, src, ok ? 8 : 0);
    }
}

// use_tma: the caller passed a tensor map of the grid (z, y, x, instance; 8-byte cells,
// box BZ x BY x 1 x CG); windows inside the grid in y and z then arrive one plane per copy
// on an mbarrier (x planes wrap freely: each is its own copy).
template <int WT, int CG>
__global__ void __launch_bounds__(256) k_interp3d_planes(InterpArgs a, const __grid_constant__ CUtensorMap map,
                                                         PlaneBox pb, int use_tma, uint32_t *status) {
    using L = Lanes2D<WT, CG>;
    constexpr int NS = kPlaneSamples;
    extern __shared__ __align__(128) float4 smem_p3[];
    __shared__ __align__(8) uint64_t bar[2];
    const Geom &g = a.g;
    const int W = WT ? WT : g.W;
    const int ns = g.ns;
    const int WX = g.tile[0] + W - 1, WY = g.tile[1] + W - 1, WZ = g.tile[2] + W - 1;
    const int cells = WY * WZ;
    const int BZ = pb.BZ, CSP = pb.BY * pb.BZ;                     // row pitch, coil stride
    const int PC = plane_elems(pb, CG);                            // float2 per plane buffer
    float2 *planes = reinterpret_cast<float2 *>(smem_p3);          // [2][PC], [coil][y][z]
    float *st_w = reinterpret_cast<float *>(planes + 2 * PC);      // [NS][48]: wx, wy, wz
    int4 *st_r = reinterpret_cast<int4 *>(st_w + NS * 48);         // [NS]: rel0, rel1, rel2, sample
    float2 *st_acc = reinterpret_cast<float2 *>(st_r + NS);        // [NS][CG]

    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    int o[3], e[3];
    tile_coords<3>(g, sub.x % g.ntiles, o, e);
    const int ws0 = o[0] - (ns - 1), ws1 = o[1] - (ns - 1), ws2 = o[2] - (ns - 1);
    const float2 *base = a.grid + ((int64_t)grp * g.n_coil + cg0) * g.G;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int c = lane % CG, q = lane / CG;
    const float rWZ = 1.f / (float)WZ, rcells = 1.f / (float)cells;
    // tensor copies for windows inside the grid in y and z; the copy starts on an even z
    const int zs = ws2 - (ws2 & 1);
    const bool tma = use_tma && ws1 >= 0 && ws1 + pb.BY <= g.nf[1] && ws2 >= 0 && zs + BZ <= g.nf[2];
    const int offz = tma ? ws2 - zs : 0;
    const uint32_t box_bytes = (uint32_t)(CSP * CG * sizeof(float2));
    if (tma && threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    uint32_t parity = 0u;  // bit b: phase parity expected next on buffer b's barrier

    // start the copy of plane px into buffer b (tensor copy by one thread, or the threads')
    auto stage = [&](int px, int b) {
        float2 *dst = planes + b * PC;
        const int gx = wrap_fast(ws0 + px, g.nf[0]);
        if (tma) {
            if (threadIdx.x == 0) {
                fence_proxy_async_smem();  // the buffer's previous readers come first
                mbar_arrive_expect_tx(&bar[b], box_bytes);
                tma_load_4d(dst, &map, zs, ws1, gx, grp * g.n_coil + cg0, &bar[b]);
            }
        } else {
            plane_copy<CG>(dst, base, g, cg0, gx, ws1, ws2, WZ, cells, BZ, CSP, rWZ, rcells);
        }
    };

    for (int base_s = 0; base_s < sub.z; base_s += NS) {
        const int n = min(NS, sub.z - base_s);
        __syncthreads();  // the previous chunk's state and planes are consumed (and the barriers set up)
        stage(0, 0);
        for (int i = threadIdx.x; i < n * 48; i += blockDim.x) {
            const int s = i / 48, k = i - s * 48, d = k >> 4, kq = k & 15;
            const float4 p = a.pts[(int64_t)sub.y + base_s + s];
            const float f = d == 0 ? p.x : (d == 1 ? p.y : p.z);
            const float b = d == 0 ? g.beta2[0] : (d == 1 ? g.beta2[1] : g.beta2[2]);
            st_w[i] = tap_weight(true, kq, W, f, ns, b);
            if (k == 0) {
                int c0[3];
                unpack_cells(3, __float_as_uint(p.w), c0[0], c0[1], c0[2]);
                int rel[3];
#pragma unroll
                for (int dd = 0; dd < 3; ++dd) {
                    int cc = c0[dd] + ns - 1;
                    cc -= cc >= g.nf[dd] ? g.nf[dd] : 0;
                    rel[dd] = cc - o[dd];
                }
                st_r[s] = make_int4(rel[0], rel[1], rel[2], (int)a.idx[(int64_t)sub.y + base_s + s]);
            }
        }
        for (int i = threadIdx.x; i < n * CG; i += blockDim.x) st_acc[i] = make_float2(0.f, 0.f);
        if (!tma) cp_async_wait_all();
        __syncthreads();

        for (int px = 0; px < WX; ++px) {
            const int b = px & 1;
            if (tma) {
                if (!mbar_wait_bounded(&bar[b], (parity >> b) & 1u) && lane == 0) atomicOr(status, kStatusTmaTimeout);
                parity ^= 1u << b;
            }
            const float2 *cur = planes + b * PC;
            // the next plane's copy runs while this one is used (its buffer was last read
            // before the previous barrier)
            if (px + 1 < WX) stage(px + 1, b ^ 1);
            for (int s = warp; s < n; s += nw) {
                const int4 r = st_r[s];
                const int kx = px - r.x;
                if ((unsigned)kx >= (unsigned)W) continue;  // warp-uniform: stencil misses this plane
                const float *w = st_w + s * 48;
                float2 at[L::KT];
#pragma unroll
                for (int t = 0; t < L::KT; ++t) at[t] = make_float2(0.f, 0.f);
                const float2 *rowbase = cur + c * CSP + r.y * BZ + r.z + offz;
                float wys[(L::WMAX + 3) & ~3];  // y weights by 16-byte broadcast loads
#pragma unroll
                for (int k4 = 0; k4 < (L::WMAX + 3) / 4; ++k4) {
                    const float4 v = *reinterpret_cast<const float4 *>(w + 16 + 4 * k4);
                    wys[4 * k4] = v.x;
                    wys[4 * k4 + 1] = v.y;
                    wys[4 * k4 + 2] = v.z;
                    wys[4 * k4 + 3] = v.w;
                }
#pragma unroll
                for (int ky = 0; ky < L::WMAX; ++ky) {
                    if (WT == 0 && ky >= W) break;
                    const float wy = wys[ky];
                    const float2 wy2 = make_float2(wy, wy);
                    const float2 *row = rowbase + ky * BZ;
#pragma unroll
                    for (int t = 0; t < L::KT; ++t) {
                        const int kz = q + t * L::NQ;
                        if (kz < W) at[t] = __ffma2_rn(wy2, row[kz], at[t]);
                    }
                }
                float ax = 0.f, ay = 0.f;
#pragma unroll
                for (int t = 0; t < L::KT; ++t) {
                    const int kz = q + t * L::NQ;
                    const float wz = kz < W ? w[32 + kz] : 0.f;
                    ax = fmaf(wz, at[t].x, ax);
                    ay = fmaf(wz, at[t].y, ay);
                }
#pragma unroll
                for (int off = CG; off < 32; off <<= 1) {
                    ax += __shfl_xor_sync(0xffffffffu, ax, off);
                    ay += __shfl_xor_sync(0xffffffffu, ay, off);
                }
                if (q == 0) {
                    const float wx = w[kx];
                    float2 &acc = st_acc[s * CG + c];
                    acc.x = fmaf(wx, ax, acc.x);
                    acc.y = fmaf(wx, ay, acc.y);
                }
            }
            if (!tma) cp_async_wait_all();
            __syncthreads();
        }

        for (int i = threadIdx.x; i < n * CG; i += blockDim.x) {
            const int s = i / CG, cc = i - s * CG;
            if (cg0 + cc < g.n_coil) {
                const uint32_t j = (uint32_t)st_r[s].w;
                float2 v = st_acc[i];
                if (a.weight) {
                    const float sw = a.weight[j];
                    v.x *= sw;
                    v.y *= sw;
                }
                a.c[(int64_t)j * a.c_elem + (int64_t)(cg0 + cc) * a.c_coil] = v;
            }
        }
    }
}

// shared memory of k_interp3d_planes, or 0 when the plane kernel does not apply
inline size_t interp3d_planes_smem_bytes(const Geom &g, int cg, int threads) {
    (void)threads;
    if (g.dim != 3 || g.W > 16 || (cg != 4 && cg != 8)) return 0;
    const PlaneBox pb = plane_box(g, cg);
    const int PC = plane_elems(pb, cg);
    if (pb.BY == 0 || PC > kPlaneMaxElems) return 0;
    return 2 * (size_t)PC * sizeof(float2) + kPlaneSamples * (48 * sizeof(float) + sizeof(int4)) +
           (size_t)kPlaneSamples * cg * sizeof(float2);
}

// --------------------------------------------------------------------------------- spread
constexpr int kSpread3dBatch = 32;

template <int WT, int CG>
__global__ void __launch_bounds__(256) k_spread3d(SpreadArgs a) {
    using L = Lanes2D<WT, CG>;
    extern __shared__ float4 smem_s3[];
    const Geom &g = a.g;
    const int TX = g.tile[0], TY = g.tile[1], TZ = g.tile[2];
    float2 *acc = reinterpret_cast<float2 *>(smem_s3);                        // [TX][TY][TZ][CG]
    float *st_w = reinterpret_cast<float *>(acc + (size_t)TX * TY * TZ * CG);  // [batch][48]: wx, wy, wz
    float2 *st_v = reinterpret_cast<float2 *>(st_w + kSpread3dBatch * 48);     // [batch][CG]
    int4 *st_r = reinterpret_cast<int4 *>(st_v + kSpread3dBatch * CG);         // [batch]: signed first taps

    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    int o[3], e[3];
    tile_coords<3>(g, sub.x % g.ntiles, o, e);
    const int W = WT ? WT : g.W;
    const int ns = g.ns;

    for (int i = threadIdx.x; i < TX * TY * TZ * CG; i += blockDim.x) acc[i] = make_float2(0.f, 0.f);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int c = lane % CG, q = lane / CG;
    const int P = (TX + nw - 1) / nw;
    const int x0 = warp * P, x1 = min(x0 + P, e[0]);

    for (int base = 0; base < sub.z; base += kSpread3dBatch) {
        const int n = min(kSpread3dBatch, sub.z - base);
        __syncthreads();
        for (int i = threadIdx.x; i < n * 48; i += blockDim.x) {
            const int s = i / 48, k = i - s * 48, d = k >> 4, kq = k & 15;
            const float4 p = a.pts[(int64_t)sub.y + base + s];
            float val = 0.f;
            if (kq < W) {
                const float f = d == 0 ? p.x : (d == 1 ? p.y : p.z);
                const float dd = f + (float)(ns - 1 - kq);
                val = exp2f(-g.beta2[d] * dd * dd);
            }
            st_w[i] = val;
            if (k == 0) {
                int c0[3];
                unpack_cells(3, __float_as_uint(p.w), c0[0], c0[1], c0[2]);
                int r[3];
#pragma unroll
                for (int dd = 0; dd < 3; ++dd) {
                    int rr = c0[dd] - o[dd];
                    rr += rr < 0 ? g.nf[dd] : 0;
                    rr -= rr > g.nf[dd] - W ? g.nf[dd] : 0;
                    r[dd] = rr;
                }
                st_r[s] = make_int4(r[0], r[1], r[2], 0);
            }
        }
        for (int i = threadIdx.x; i < n * CG; i += blockDim.x) {
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
            st_v[i] = v;
        }
        __syncthreads();

        for (int s = 0; s < n; ++s) {
            const int4 r = st_r[s];
            const int xl = max(x0, r.x), xh = min(x1, r.x + W);
            if (xl >= xh) continue;
            const int yl = max(0, r.y), yh = min(e[1], r.y + W);
            if (yl >= yh) continue;
            const float2 v = st_v[s * CG + c];
            const float *w = st_w + s * 48;
            if constexpr (CG == 1) {
                // one coil: lane (yo, kz) takes z tap kz on every other y row from yl + yo, so
                // 32 lanes cover 16 tap slots on two rows at once
                const int kz = lane & 15, yo = lane >> 4;
                const int z = r.z + kz;
                const bool zok = kz < W && (unsigned)z < (unsigned)e[2];
                const float wz1 = zok ? w[32 + kz] : 0.f;
                const float2 vz = make_float2(wz1 * v.x, wz1 * v.y);
                for (int x = xl; x < xh; ++x) {
                    const float wx = w[x - r.x];
                    float2 *rowp = acc + ((size_t)x * TY + yl + yo) * TZ + z;
                    for (int y = yl + yo; y < yh; y += 2, rowp += 2 * TZ) {
                        const float wxy = wx * w[16 + y - r.y];
                        if (zok) *rowp = __ffma2_rn(make_float2(wxy, wxy), vz, *rowp);
                    }
                }
            } else {
                float wz[L::KT];
                int lz[L::KT];
#pragma unroll
                for (int t = 0; t < L::KT; ++t) {
                    const int kz = q + t * L::NQ;
                    const int z = r.z + kz;
                    const bool ok = kz < W && (unsigned)z < (unsigned)e[2];
                    wz[t] = ok ? w[32 + kz] : 0.f;
                    lz[t] = ok ? z : -1;
                }
                for (int x = xl; x < xh; ++x) {
                    const float wx = w[x - r.x];
                    for (int y = yl; y < yh; ++y) {
                        const float wxy = wx * w[16 + y - r.y];
                        float2 *rowp = acc + ((size_t)x * TY + y) * TZ * CG + c;
#pragma unroll
                        for (int t = 0; t < L::KT; ++t) {
                            if (lz[t] >= 0) {
                                float2 *cell = rowp + (size_t)lz[t] * CG;
                                const float ww = wxy * wz[t];
                                *cell = __ffma2_rn(make_float2(ww, ww), v, *cell);
                            }
                        }
                    }
                }
            }
        }
    }
    __syncthreads();

    const bool split = (sub.w & kSplitFlag) != 0;
    const int ecell = e[0] * e[1] * e[2];
    for (int i = threadIdx.x; i < ecell * CG; i += blockDim.x) {
        const int cc = i % CG, cell = i / CG;
        if (cg0 + cc >= g.n_coil) continue;
        const int lz = cell % e[2], ly = (cell / e[2]) % e[1], lx = cell / (e[2] * e[1]);
        const float2 val = acc[(((size_t)lx * TY + ly) * TZ + lz) * CG + cc];
        float2 *dst = a.grid + ((int64_t)grp * g.n_coil + cg0 + cc) * g.G +
                      ((int64_t)(o[0] + lx) * g.nf[1] + (o[1] + ly)) * g.nf[2] + (o[2] + lz);
        if (split) {
            atomicAdd(&dst->x, val.x);
            atomicAdd(&dst->y, val.y);
        } else {
            *dst = val;
        }
    }
}

// ------------------------------------------------------------------ spread, register tile
// For 4 or 8 coils per block: warp w owns the 4 (x, y) rows  rho = 4w .. 4w+3  of the tile
// (TY a multiple of 4, so they share x and have consecutive y) and lane (c, q) holds z
// cells q, q + NQ, q + 2NQ, q + 3NQ of coil c in registers: tile (4*warps/TY) x TY x 4*NQ.
// No shared-memory read-modify-write.
//
// Staging as in k_spread2d_reg (double-buffered batches of 32, one barrier per batch):
// warp 0 stages the weight of every tile x plane and builds the ordered per-warp sample
// lists (the stencil reaches the warp's x plane and one of its 4 y rows), warp 1 the
// weight of every y row, warp 2 of every z column ([q][k] for column q + k*NQ), the other
// warps gather the coil values.  Per listed sample a warp loads its plane weight, its 4
// row weights and its 4 column weights, folds the plane and column weights into the coil
// value (10 multiplies) and issues 16 packed FMAs.
//
// KAHAN: the instance for the subproblems flagged kDenseFlag (tiles above the dense-sample
// threshold: the k-space centre of radial data, where a cell sums thousands of terms).
// Blocked Kahan summation: each staged batch (32 samples) accumulates plainly into a
// register partial, and the partial is added once per batch to the cell's total with a
// compensation term (the low-order part lost by that addition is carried into the next
// one); the flush writes total - compensation.  The rounding error then grows with the
// batch length rather than the tile's sample count, at 16 compensated additions per
// lane per batch.  The plain instance skips dense subproblems and the Kahan instance the
// others, so the two launches together cover every subproblem once.
__device__ __forceinline__ void kahan_add(float2 &s, float2 &cmp, float2 v) {
    const float yx = v.x - cmp.x, yy = v.y - cmp.y;
    const float tx = s.x + yx, ty = s.y + yy;
    cmp.x = (tx - s.x) - yx;
    cmp.y = (ty - s.y) - yy;
    s.x = tx;
    s.y = ty;
}

template <int WT, int CG, bool KAHAN>
__global__ void __launch_bounds__(256) k_spread3d_reg(SpreadArgs a) {
    constexpr int NQ = 32 / CG;
    constexpr int B = kRegBatch;
    extern __shared__ float4 smem_r3[];
    if (((a.subs[blockIdx.x].w & kDenseFlag) != 0) != KAHAN) return;  // the other launch's subproblem
    const Geom &g = a.g;
    const int TX = g.tile[0], TY = g.tile[1], TZ = g.tile[2];
    // per staged sample: y rows [0, TY), z columns [TY, TY + TZ) as [q][k], x planes after
    // them; the stride is padded to a multiple of 4 (16-byte loads) plus a bank offset
    const int TWP = reg_stride(TY + TZ + 4 * ((TX + 3) / 4));
    const int nw = blockDim.x >> 5;
    float *st_w = reinterpret_cast<float *>(smem_r3);                  // [2][B][TWP]
    float2 *st_v = reinterpret_cast<float2 *>(st_w + 2 * B * TWP);     // [2][B][CG]
    int *st_cnt = reinterpret_cast<int *>(st_v + 2 * B * CG);          // [2][8]
    uint8_t *st_list = reinterpret_cast<uint8_t *>(st_cnt + 16);       // [2][8][B]

    const int4 sub = a.subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int grp = sub.x / g.ntiles;
    int o[3], e[3];
    tile_coords<3>(g, sub.x % g.ntiles, o, e);
    const int W = WT ? WT : g.W;
    const int ns = g.ns;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = lane % CG, q = lane / CG;
    const int rho0 = warp * kRegRows;
    const int xw = rho0 / TY, y0 = rho0 - xw * TY;
    float2 acc[kRegRows][kRegCols];
    // Kahan instance: compensated totals and their compensation terms
    float2 tot[KAHAN ? kRegRows : 1][KAHAN ? kRegCols : 1], cmp[KAHAN ? kRegRows : 1][KAHAN ? kRegCols : 1];
#pragma unroll
    for (int r = 0; r < kRegRows; ++r)
#pragma unroll
        for (int k = 0; k < kRegCols; ++k) acc[r][k] = make_float2(0.f, 0.f);
    if constexpr (KAHAN) {
#pragma unroll
        for (int r = 0; r < kRegRows; ++r)
#pragma unroll
            for (int k = 0; k < kRegCols; ++k) {
                tot[r][k] = make_float2(0.f, 0.f);
                cmp[r][k] = make_float2(0.f, 0.f);
            }
    }

    for (int base = 0, buf = 0; base < sub.z; base += B, buf ^= 1) {
        const int n = min(B, sub.z - base);
        if (warp < 3) {
            const bool ok = lane < n;
            float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
            int r[3] = {0, 0, 0};
            if (ok) {
                p = a.pts[(int64_t)sub.y + base + lane];
                int c0[3];
                unpack_cells(3, __float_as_uint(p.w), c0[0], c0[1], c0[2]);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    int rr = c0[d] - o[d];
                    rr += rr < 0 ? g.nf[d] : 0;
                    rr -= rr > g.nf[d] - W ? g.nf[d] : 0;
                    r[d] = rr;
                }
            }
            // warp 0: x planes (+ lists), warp 1: y rows, warp 2: z columns; 16-byte stores
            float *dst = st_w + (buf * B + lane) * TWP;
            if (warp == 0) {
                const float b = g.beta2[0];
                for (int k4 = 0; k4 < TX; k4 += 4)  // planes past TX get harmless unused weights
                    *reinterpret_cast<float4 *>(dst + TY + TZ + k4) =
                        make_float4(tap_weight(ok, k4 - r[0], W, p.x, ns, b), tap_weight(ok, k4 + 1 - r[0], W, p.x, ns, b),
                                    tap_weight(ok, k4 + 2 - r[0], W, p.x, ns, b),
                                    tap_weight(ok, k4 + 3 - r[0], W, p.x, ns, b));
            } else if (warp == 1) {
                const float b = g.beta2[1];
                for (int k4 = 0; k4 < TY; k4 += 4)
                    *reinterpret_cast<float4 *>(dst + k4) =
                        make_float4(tap_weight(ok, k4 - r[1], W, p.y, ns, b), tap_weight(ok, k4 + 1 - r[1], W, p.y, ns, b),
                                    tap_weight(ok, k4 + 2 - r[1], W, p.y, ns, b),
                                    tap_weight(ok, k4 + 3 - r[1], W, p.y, ns, b));
            } else {
                const float b = g.beta2[2];
#pragma unroll
                for (int cq = 0; cq < NQ; ++cq)  // columns cq + k*NQ, k = 0..3
                    *reinterpret_cast<float4 *>(dst + TY + cq * 4) =
                        make_float4(tap_weight(ok, cq - r[2], W, p.z, ns, b),
                                    tap_weight(ok, cq + NQ - r[2], W, p.z, ns, b),
                                    tap_weight(ok, cq + 2 * NQ - r[2], W, p.z, ns, b),
                                    tap_weight(ok, cq + 3 * NQ - r[2], W, p.z, ns, b));
            }
            if (warp == 0) {
                for (int w = 0; w < nw; ++w) {
                    const int wx = (w * kRegRows) / TY, wy0 = w * kRegRows - wx * TY;
                    const bool hit = ok && (unsigned)(wx - r[0]) < (unsigned)W && r[1] < wy0 + kRegRows &&
                                     r[1] + W > wy0;
                    const unsigned m = __ballot_sync(0xffffffffu, hit);
                    if (hit) st_list[(buf * 8 + w) * B + __popc(m & lanemask_lt(lane))] = (uint8_t)lane;
                    if (lane == 0) st_cnt[buf * 8 + w] = __popc(m);
                }
            }
        } else {
            for (int i = threadIdx.x - 96; i < n * CG; i += blockDim.x - 96) {
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
        __syncthreads();  // one barrier per batch: the other buffer is free (double buffering)

        const int cnt = st_cnt[buf * 8 + warp];
        const uint8_t *lst = st_list + (buf * 8 + warp) * B;
        for (int i = 0; i < cnt; ++i) {
            const int s = buf * B + lst[i];
            const float *w = st_w + s * TWP;
            const float2 v0 = st_v[s * CG + c];
            const float wx = w[TY + TZ + xw];
            const float2 v = make_float2(wx * v0.x, wx * v0.y);
            const float4 wz = *reinterpret_cast<const float4 *>(w + TY + q * 4);
            const float4 wy = *reinterpret_cast<const float4 *>(w + y0);
            const float2 u[kRegCols] = {make_float2(wz.x * v.x, wz.x * v.y), make_float2(wz.y * v.x, wz.y * v.y),
                                        make_float2(wz.z * v.x, wz.z * v.y), make_float2(wz.w * v.x, wz.w * v.y)};
            const float wyr[kRegRows] = {wy.x, wy.y, wy.z, wy.w};
#pragma unroll
            for (int rr = 0; rr < kRegRows; ++rr) {
                const float2 wy2 = make_float2(wyr[rr], wyr[rr]);
#pragma unroll
                for (int k = 0; k < kRegCols; ++k) acc[rr][k] = __ffma2_rn(wy2, u[k], acc[rr][k]);
            }
        }
        if constexpr (KAHAN) {
            // fold this batch's partial sums into the compensated totals
#pragma unroll
            for (int rr = 0; rr < kRegRows; ++rr)
#pragma unroll
                for (int k = 0; k < kRegCols; ++k) {
                    kahan_add(tot[rr][k], cmp[rr][k], acc[rr][k]);
                    acc[rr][k] = make_float2(0.f, 0.f);
                }
        }
    }
    if constexpr (KAHAN) {
#pragma unroll
        for (int rr = 0; rr < kRegRows; ++rr)
#pragma unroll
            for (int k = 0; k < kRegCols; ++k)
                acc[rr][k] = make_float2(tot[rr][k].x - cmp[rr][k].x, tot[rr][k].y - cmp[rr][k].y);
    }

    if (cg0 + c >= g.n_coil || xw >= e[0]) return;
    const bool split = (sub.w & kSplitFlag) != 0;
    float2 *dstc = a.grid + ((int64_t)grp * g.n_coil + cg0 + c) * g.G;
#pragma unroll
    for (int rr = 0; rr < kRegRows; ++rr) {
        const int ly = y0 + rr;
        if (ly >= e[1]) break;
#pragma unroll
        for (int k = 0; k < kRegCols; ++k) {
            const int lz = q + k * NQ;
            if (lz >= e[2]) continue;
            float2 *dst = dstc + ((int64_t)(o[0] + xw) * g.nf[1] + (o[1] + ly)) * g.nf[2] + (o[2] + lz);
            if (split) {
                atomicAdd(&dst->x, acc[rr][k].x);
                atomicAdd(&dst->y, acc[rr][k].y);
            } else {
                *dst = acc[rr][k];
            }
        }
    }
}

inline size_t spread3d_reg_smem_bytes(const Geom &g, int cg) {
    const int twp = reg_stride(g.tile[1] + g.tile[2] + 4 * ((g.tile[0] + 3) / 4));
    return 2 * ((size_t)kRegBatch * twp * sizeof(float) + (size_t)kRegBatch * cg * sizeof(float2)) +
           16 * sizeof(int) + 2 * 8 * kRegBatch;
}

inline size_t spread3d_smem_bytes(const Geom &g, int cg) {
    return (size_t)g.tile[0] * g.tile[1] * g.tile[2] * cg * sizeof(float2) + kSpread3dBatch * 48 * sizeof(float) +
           (size_t)kSpread3dBatch * cg * sizeof(float2) + kSpread3dBatch * sizeof(int4);
}

inline size_t interp3d_smem_bytes(const Geom &g, int cg) {
    return (size_t)(g.tile[0] + g.W - 1) * (g.tile[1] + g.W - 1) * (g.tile[2] + g.W - 1) * cg * sizeof(float2);
}

}  // namespace gbn
