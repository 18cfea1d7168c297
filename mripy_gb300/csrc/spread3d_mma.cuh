// Spread (type-1 gridding) of 8 coils on the tensor cores: k_spread_mma<D, WT, KAHAN>, 3-D
// (the default for 8 coils) and 2-D (selectable).
//
// The adjoint gridding of one tile is a sum of outer products over its samples s:
//     G[x, y, z, c] = sum_s wx_s[x] wy_s[y] wz_s[z] v_s[c]
// and with the separable weights split between the two operands it is a GEMM with the
// samples as its K dimension:
//     D[(y, z), (x, c, re/im)] = sum_s A[(y, z), s] * B[s, (x, c, re/im)]
//     A[(y, z), s] = wy_s[y] wz_s[z]                      (M = 8 x 16 = 128 cells)
//     B[s, (x, c, ri)] = wx_s[x] * (re, im)(v_s[c])       (N = 4 x 8 x 2 = 64)
// on tiles of 4 x 8 x 16 cells (2-D: tiles of 8 x 16 cells, the two grid axes in the roles
// of y and z, and B the coil values alone, N = 16).  The accumulator D lives in tensor memory
// (TMEM); A is built in TMEM (tcgen05.st), B in shared memory (K-major, 128-byte swizzle);
// one tcgen05.mma.kind::tf32 covers 8 samples.  Each FP32 operand is split as x = hi + lo
// with hi on the TF32 grid, and three MMAs (hi*hi + hi*lo + lo*hi) give products within
// ~1e-6 of FP32 (the lo*lo term, below 2^-22 relative, is left out).  The tensor core
// evaluates the whole tile for every sample (a 12-tap stencil covers ~22 % of a 4 x 8 x 16
// tile on average) but needs no per-cell instruction: the CUDA cores build 192 operand
// values per (sample, tile) pair instead of issuing the stencil's FMAs.
//
// One (work item, coil group) unit per block; 3 loader warps, NB builder warps (8 in the
// plain instance, 16 in the compensated one) and 1 MMA warp:
// * the loader warps fill a ring of kMmaSlots 32-sample batches (loader l: batches l, l + 3,
//   ...; the sample indices of batch l are read before the block's set-up): per sample and
//   dimension the first tap's tile plane and the distance of plane 0, and the 8 coil values
//   times the optional density weight ([coil][sample]); `full` / `empty` mbarriers per slot.
// * the builder warps first compute the batch's tile-plane weights per sample together
//   (stored [plane][sample]; a named barrier among them), then turn the batch into the MMA
//   operands: warp b writes A's hi and lo parts for the 32 TMEM lanes of its quarter (b % 4)
//   and 128 / NB of the 32 samples, and N / NB of B's rows into shared memory; two operand
//   buffers, the one of batch t reused by batch t + 2 after the MMAs of batch t completed
//   (`done` mbarrier, signalled by tcgen05.commit).  After the last batch they read D back
//   (tcgen05.ld) and write the tile.
// * the MMA warp allocates TMEM, and its lane 0 issues 12 MMAs per batch once the builders
//   arrived on the buffer's `ops` mbarrier, then commits to the buffer's `done` mbarrier.
// Summation: the tensor core's FP32 accumulation rounds less carefully than FP32 adds (its
// error grew with the number of accumulated MMAs: 1.6e-6 relative to the FP32 kernel with
// 1024-sample work items, 4.9e-6 with 8192, on the 3-D radial workload), so the plain
// instance sums groups of kMmaGroup batches (256 samples, 96 MMAs) only; the builders then
// add the accumulator into a running sum S in TMEM with FP32 adds before the next group's
// first MMA overwrites it.  The compensated instance (KAHAN: the 3-D dense, k-space-centre
// units, one block per SM) drains every batch's accumulator (two of them alternate) into a
// group sum G with FP32 adds and folds G into a Kahan-compensated sum S, C in TMEM every
// kMmaGroup batches (measured against a Kahan add per batch: the same centre-cell error,
// 3.8e-7, in 1.5 % less time).  The order is fixed for a given trajectory and tiling.
//
// Every wait is bounded (kTmaWaitLimit probes); one that gives up sets kStatusSpreadTimeout
// in the plan's status word and goes on, so no launch can hang.  The plain instance runs a
// block per unit and leaves the dense ones at once; the compensated instance runs a block
// per dense unit only, through the plan's list of dense subproblems.
#pragma once

#include "common.cuh"
#include "grid2d_kernels.cuh"
#include "grid3d_kernels.cuh"
#include "spread3d_cube.cuh"
#include "tc.cuh"

namespace gbn {

constexpr int kMmaTX = 4, kMmaTY = 8, kMmaTZ = 16;  // the tile this kernel takes
constexpr int kMmaM = kMmaTY * kMmaTZ;              // 128 cells (y, z): one TMEM lane each
constexpr int kMmaN = kMmaTX * 16;                  // 64 columns (x, coil, re/im)
constexpr int kMmaBatch = 32;                       // samples per batch: one 128-byte K row
constexpr int kMmaSlots = 8;                        // staged batches
#ifndef GBN_MMA_LOADERS
#define GBN_MMA_LOADERS 3
#endif
constexpr int kMmaLoaders = GBN_MMA_LOADERS;
// builder warps: 8 in the plain instance (two blocks per SM, registers), 16 in the
// compensated one (one block per SM: more warps hide its latencies)
template <bool KAHAN> constexpr int mma_builders() { return KAHAN ? 16 : 8; }
template <bool KAHAN> constexpr int mma_threads() { return 32 * (mma_builders<KAHAN>() + kMmaLoaders + 1); }
constexpr uint32_t kMmaTmemCols = 256;              // A (hi, lo) x 2 buffers: 0..127; D, S: 128..255
constexpr uint32_t kMmaColD = 128;                  // the MMAs' accumulator
constexpr uint32_t kMmaColS = 192;                  // the running sum of the drained accumulators (3-D)
// the compensated instance: two accumulators D (batch k in D[k % 2]), the running sum S, its
// Kahan compensation C and the current group's FP32 sum G; one block per SM
constexpr uint32_t kMmaTmemColsK = 512;
constexpr uint32_t kMmaColSK = 256, kMmaColCK = 320, kMmaColGK = 384;
constexpr int kMmaGroup = 8;                        // batches the tensor core sums before a drain
constexpr int kMmaWS = 36;  // floats per staged [tap] row of 32 samples: 16-byte aligned, 4-bank skew

// shared memory, bytes from a 1024-byte aligned base
constexpr uint32_t kMmaBOp = kMmaN * 128;                               // one B operand: 64 rows x 128 B
constexpr uint32_t kMmaStWx = 0;                                        // [TX][kMmaWS] floats
constexpr uint32_t kMmaStWy = kMmaStWx + 4 * kMmaTX * kMmaWS;           // [TY][kMmaWS]
constexpr uint32_t kMmaStWz = kMmaStWy + 4 * kMmaTY * kMmaWS;           // [TZ][kMmaWS]
constexpr uint32_t kMmaStV = kMmaStWz + 4 * kMmaTZ * kMmaWS;            // [8 coils][32] float2
constexpr uint32_t kMmaStD0 = kMmaStV + 8 * 8 * kMmaBatch;              // [3][32] float: d of tap 0
constexpr uint32_t kMmaStR = kMmaStD0 + 4 * 3 * kMmaBatch;              // [3][32] int: first tap's cell
constexpr uint32_t kMmaSlotBytes = kMmaStR + 4 * 3 * kMmaBatch;
constexpr uint32_t kMmaStageOff = 4 * kMmaBOp;                          // after B (hi, lo) x 2 buffers
constexpr uint32_t kMmaBarOff = kMmaStageOff + kMmaSlots * kMmaSlotBytes;
constexpr uint32_t kMmaBars = 2 * kMmaSlots + 4;                        // full, empty, ops[2], done[2]
// + the TMEM address word and the alignment slack.  Above a third of the SM's 228 KB, so at
// most two blocks (2 x 256 TMEM columns) share an SM and tcgen05.alloc never waits.
constexpr size_t kMmaSmemBytes = kMmaBarOff + 8 * kMmaBars + 16 + 1024;
static_assert(kMmaSmemBytes > 228 * 1024 / 3, "two blocks per SM at most");
// the compensated instance asks for more than half the SM's shared memory: one block per SM
// holds all 512 TMEM columns
constexpr size_t kMmaSmemBytesK = 116 * 1024;
static_assert(kMmaSmemBytesK > 228 * 1024 / 2 && kMmaSmemBytesK >= kMmaSmemBytes, "one block per SM");
static_assert(kMmaStV % 16 == 0 && kMmaSlotBytes % 16 == 0, "16-byte aligned staging");
constexpr int kMmaTaps = kMmaTX + kMmaTY + kMmaTZ;  // 28 tile-plane weights per sample

// The tile of each dimension: M = TY x TZ = 128 cells of grid dimensions (DY, DZ), N = NX
// planes along grid dimension 0 (3-D only) x 8 coils x re/im.  3-D: 4 x 8 x 16 cells,
// N = 64.  2-D: 8 x 16 cells, N = 16 (no plane weight: B is the coil values themselves).
template <int D> struct MmaTile;
template <> struct MmaTile<3> {
    static constexpr int NX = 4, DY = 1, DZ = 2, TAPS = kMmaTX + kMmaTY + kMmaTZ;
};
template <> struct MmaTile<2> {
    static constexpr int NX = 1, DY = 0, DZ = 1, TAPS = kMmaTY + kMmaTZ;
};
template <int D> constexpr int mma_n() { return MmaTile<D>::NX * 16; }

// 2^x (PTX ex2.approx, flushing subnormal results to zero: the Gaussian's smallest weight
// inside the stencil is ~eps, far above the subnormal range)
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Two products x = a * b (one packed FP32x2 multiply) split as x = hi + lo: hi rounded to
// the TF32 grid (11 significant bits; ties away from zero, by integer arithmetic on the bit
// pattern), lo = x - hi exactly (one packed subtraction).  The tensor core reads lo's top 11
// significant bits.  (Dekker's split t = x (2^13 + 1), hi = t - (t - x) in packed FP32x2
// arithmetic was measured on GB300 to return hi = x, lo = 0, so it is not used.)
__device__ __forceinline__ float tf32_round_bits(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
// (Rounding lo to the TF32 grid as well and adding the lo * lo MMA left the compensated
// instance's centre-cell error unchanged, 3.9e-7 against 3.8e-7 on the 3-D radial test
// data, and cost 0.09 ms of 6.0 on the 3-D radial workload: the tensor core's own FP32
// accumulation within a batch dominates, so neither is done.)
__device__ __forceinline__ void tf32_split2(float2 a, float2 b, float2 &hi, float2 &lo) {
    const float2 x = __fmul2_rn(a, b);
    hi = make_float2(tf32_round_bits(x.x), tf32_round_bits(x.y));
    lo = __fadd2_rn(x, make_float2(-hi.x, -hi.y));
}

// S (+)= D over this thread's lane and the N / 2 columns of half hk; `first`: S = D.  D is
// at column kMmaColD, S right after it (N columns each).
template <int N>
__device__ __forceinline__ void mma_drain(uint32_t tl, int hk, bool first) {
    constexpr uint32_t kColS = kMmaColD + N;
    if constexpr (N == 64) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t col = 32u * hk + 16u * h;
            float d[16], s[16];
            tmem_ld_x16(tl + kMmaColD + col, d);
            if (!first) {
                tmem_ld_x16(tl + kColS + col, s);
                tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) d[i] += s[i];
            } else {
                tmem_wait_ld();
            }
            tmem_st_x16(tl + kColS + col, d);
        }
    } else {
        static_assert(N == 16, "N is 64 (3-D) or 16 (2-D)");
        const uint32_t col = 8u * hk;
        float d[8], s[8];
        tmem_ld_x8(tl + kMmaColD + col, d);
        if (!first) {
            tmem_ld_x8(tl + kColS + col, s);
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 8; ++i) d[i] += s[i];
        } else {
            tmem_wait_ld();
        }
        tmem_st_x8(tl + kColS + col, d);
    }
}

// S, C (+)= D[col_d] with Kahan compensation over this thread's lane and NCH 16-column
// chunks from column col0 (scalar FP32 operations); `first`: S = D, C = 0
template <int NCH>
__device__ __forceinline__ void mma_drain_kahan(uint32_t tl, uint32_t col0, uint32_t col_d, bool first) {
#pragma unroll
    for (int h = 0; h < NCH; ++h) {
        const uint32_t col = col0 + 16u * h;
        float d[16], s[16], c[16];
        tmem_ld_x16(tl + col_d + col, d);
        if (first) {
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 16; ++i) c[i] = 0.f;
            tmem_st_x16(tl + kMmaColSK + col, d);
        } else {
            tmem_ld_x16(tl + kMmaColSK + col, s);
            tmem_ld_x16(tl + kMmaColCK + col, c);
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const float y = d[i] - c[i];
                const float t = s[i] + y;
                c[i] = (t - s[i]) - y;
                s[i] = t;
            }
            tmem_st_x16(tl + kMmaColSK + col, s);
        }
        tmem_st_x16(tl + kMmaColCK + col, c);
    }
}

// G (+)= D[col_d] over this thread's lane and NCH 16-column chunks from column col0, G at
// kMmaColGK; `first`: G = D
template <int NCH>
__device__ __forceinline__ void mma_drain_group(uint32_t tl, uint32_t col0, uint32_t col_d, bool first) {
#pragma unroll
    for (int h = 0; h < NCH; ++h) {
        const uint32_t col = col0 + 16u * h;
        float d[16], gs[16];
        tmem_ld_x16(tl + col_d + col, d);
        if (!first) {
            tmem_ld_x16(tl + kMmaColGK + col, gs);
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 16; ++i) d[i] += gs[i];
        } else {
            tmem_wait_ld();
        }
        tmem_st_x16(tl + kMmaColGK + col, d);
    }
}

// compensated instance: batch j's accumulator D[col_d] into the group sum G; when batch j
// starts a new group of kMmaGroup batches, the last group's G is first folded into the
// Kahan-compensated S, C
template <int NCH>
__device__ __forceinline__ void mma_drain_batch_k2(uint32_t tl, uint32_t col0, uint32_t col_d, int j) {
    if (j % kMmaGroup == 0 && j > 0) {
        mma_drain_kahan<NCH>(tl, col0, kMmaColGK, j == kMmaGroup);
        tmem_wait_st();
    }
    mma_drain_group<NCH>(tl, col0, col_d, j % kMmaGroup == 0);
}

// Dimension D (3: 4 x 8 x 16 tiles, N = 64; 2: 8 x 16 tiles, N = 16).  One kernel template
// rather than a device function behind per-dimension kernels: the arguments stay in the
// parameter space (an inlined copy of them cost registers and 4.5 % of the 3-D time).
template <int D, int WT, bool KAHAN>
__global__ void __launch_bounds__(mma_threads<KAHAN>(), KAHAN ? 1 : 2) k_spread_mma(SpreadArgs a, uint32_t *status, int n_cg) {
    constexpr int NB = mma_builders<KAHAN>();  // builder warps
    constexpr int WM = NB + kMmaLoaders;       // the MMA warp's index
    constexpr int SPW = 128 / NB;              // A: samples of the batch per builder warp (16 or 8)
    constexpr int RPW = mma_n<D>() / NB;       // B: rows per builder warp
    constexpr int CPW = 256 / NB;              // accumulator columns per builder warp (3-D)
    using T = MmaTile<D>;
    constexpr int N = mma_n<D>();
    constexpr uint32_t kBOp = N * 128;  // one B operand: N rows x 128 B
    constexpr uint32_t kCols = KAHAN ? kMmaTmemColsK : kMmaTmemCols;
    constexpr int B = kMmaBatch;
    constexpr int CG = 8;
    static_assert(!KAHAN || D == 3, "dense tiles are a 3-D notion");
    extern __shared__ unsigned char smem_mma_raw[];
    unsigned char *sm = smem_mma_raw + ((1024u - (smem_addr(smem_mma_raw) & 1023u)) & 1023u);
    unsigned char *opB = sm;  // [buf][hi, lo][N rows x 128 B], SW128
    unsigned char *stage = sm + kMmaStageOff;
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + kMmaBarOff);
    uint64_t *empty = full + kMmaSlots;
    uint64_t *ops = empty + kMmaSlots;
    uint64_t *done = ops + 2;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 2);

    const Geom &g = a.g;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = WT ? WT : g.W;

    // the plain instance runs a block per unit, the compensated one a block per dense unit
    // (through the list of dense subproblems); a block whose unit is of the other kind leaves
    // before it takes TMEM (all its threads alike)
    const int64_t unit = KAHAN ? (int64_t)a.dense_subs[blockIdx.x / n_cg] * n_cg + blockIdx.x % n_cg
                               : (int64_t)blockIdx.x;
    int4 sub;
    if (!cube_unit(a.subs, unit, n_cg, KAHAN, sub)) return;
    // a loader warp's first sample indices (its first batch: k = loader index), read before
    // the set-up below so that their latency overlaps it
    const int64_t stride = max(1, sub.w >> kStrideShift);  // interleaved item of a split tile
    uint32_t j0 = 0;
    if (warp >= NB && warp < WM && (warp - NB) * B + lane < sub.z)
        j0 = a.idx[(int64_t)sub.y + (int64_t)((warp - NB) * B + lane) * stride];

    if (warp == WM) {
        tmem_alloc(tslot, kCols);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < kMmaSlots; ++k) {
            mbar_init(&full[k], 32);                  // the loader warp, every lane
            mbar_init(&empty[k], NB * 32);  // every builder lane
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&ops[b], NB * 32);
            mbar_init(&done[b], 1);                   // tcgen05.commit
        }
        fence_barrier_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;

    {
        const int nb = (sub.z + B - 1) / B;
        const int cg0 = (int)(unit % n_cg) * CG;

        if (warp >= NB && warp < WM) {
            // ------------------------------------------------------------ loader warp
            int o[3], e[3];
            tile_coords<D>(g, sub.x % g.ntiles, o, e);
            const int lw = warp - NB;
            const int ns = g.ns;
            for (int k = lw; k < nb; k += kMmaLoaders) {
                const int slot = k % kMmaSlots;
                const int n = min(B, sub.z - k * B);
                const bool ok = lane < n;
                float4 pt = make_float4(0.f, 0.f, 0.f, 0.f);
                uint32_t j = 0;
                if (ok) {
                    j = k == lw ? j0 : a.idx[(int64_t)sub.y + (int64_t)(k * B + lane) * stride];
                    pt = a.pts_by_sample[j];
                }
                float sw = 1.f;
                if (ok && a.weight) sw = a.weight[j];
                float2 v[CG];
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
                    unpack_cells(D, __float_as_uint(pt.w), c0[0], c0[1], c0[2]);
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        int rr = c0[d] - o[d];
                        rr += rr < 0 ? g.nf[d] : 0;
                        rr -= rr > g.nf[d] - W ? g.nf[d] : 0;
                        r[d] = rr;
                    }
                }
                // the slot's previous batch must be released by every builder lane
                if (k >= kMmaSlots &&
                    !mbar_wait_bounded(&empty[slot], (uint32_t)((k / kMmaSlots - 1) & 1)) && lane == 0)
                    atomicOr(status, kStatusSpreadTimeout);
                unsigned char *sl = stage + (size_t)slot * kMmaSlotBytes;
                // per grid dimension: the distance of tile plane 0 from the sample (plane t:
                // d0 - t) and the plane of the first tap; a lane without a sample gets a first
                // tap no plane reaches, so all its weights are 0
                float *d0 = reinterpret_cast<float *>(sl + kMmaStD0);
                int *rs = reinterpret_cast<int *>(sl + kMmaStR);
                d0[lane] = pt.x + (float)(ns - 1 + r[0]);
                d0[B + lane] = pt.y + (float)(ns - 1 + r[1]);
                rs[lane] = ok ? r[0] : -(1 << 20);
                rs[B + lane] = ok ? r[1] : -(1 << 20);
                if constexpr (D == 3) {
                    d0[2 * B + lane] = pt.z + (float)(ns - 1 + r[2]);
                    rs[2 * B + lane] = ok ? r[2] : -(1 << 20);
                }
                float2 *vs = reinterpret_cast<float2 *>(sl + kMmaStV);
#pragma unroll
                for (int cc = 0; cc < CG; ++cc) vs[cc * B + lane] = v[cc];
                mbar_arrive(&full[slot]);
            }
        } else if (warp == WM) {
            // ------------------------------------------------------------ MMA warp
            if (lane == 0) {
                constexpr uint32_t idesc = tc_idesc_tf32(kMmaM, N);
                const uint32_t b0 = smem_addr(opB);
                for (int k = 0; k < nb; ++k) {
                    const int buf = k & 1;
                    if (!mbar_wait_bounded(&ops[buf], (uint32_t)((k >> 1) & 1))) atomicOr(status, kStatusSpreadTimeout);
                    tc_fence_after();
                    const uint32_t ah = tbase + 64u * buf, al = ah + 32u;
                    const uint32_t d = tbase + kMmaColD + (KAHAN ? 64u * buf : 0u);
                    // K step jk starts 32 jk bytes further: + 2 jk in the descriptor's address
                    // field (16-byte units; shared addresses stay far below its 14-bit range)
                    const uint64_t dbh = tc_desc_sw128(b0 + 2u * buf * kBOp), dbl = tc_desc_sw128(b0 + (2u * buf + 1u) * kBOp);
                    // plain: a group's first MMA starts D afresh; compensated: every batch's
                    const uint32_t acc0 = KAHAN ? 0u : (uint32_t)((k % kMmaGroup) != 0);
#pragma unroll
                    for (int jk = 0; jk < B / 8; ++jk) {
                        const uint64_t xh = dbh + (uint64_t)(2 * jk), xl = dbl + (uint64_t)(2 * jk);
                        tc_mma_tf32_ts(d, ah + 8u * jk, xh, idesc, jk == 0 ? acc0 : 1u);
                        tc_mma_tf32_ts(d, ah + 8u * jk, xl, idesc, 1u);
                        tc_mma_tf32_ts(d, al + 8u * jk, xh, idesc, 1u);
                    }
                    tc_commit(&done[buf]);
                }
            }
            __syncwarp();
        } else {
            // ------------------------------------------------------------ builder warp
            // warp (q, hk): TMEM quarter q; A for samples SPW hk .. SPW hk + SPW - 1 of a batch;
            // B rows RPW warp .. (3-D: x plane bx, coils bc0 .. bc0 + RPW / 2 - 1); the
            // accumulator's columns CPW hk .. (3-D)
            const int q = warp & 3, hk = warp >> 2;
            const int m = 32 * q + lane, y = m >> 4, z = m & 15;  // tile cell (y, z) of TMEM lane m
            const int bx = (RPW * warp) >> 4, bc0 = ((RPW * warp) & 15) >> 1;
            const uint32_t tl = tmem_lane_base(tbase, q);
            for (int k = 0; k < nb; ++k) {
                const int slot = k % kMmaSlots, buf = k & 1;
                if (!mbar_wait_bounded(&full[slot], (uint32_t)((k / kMmaSlots) & 1)) && lane == 0)
                    atomicOr(status, kStatusSpreadTimeout);
                {
                    // the batch's tile-plane weights per sample (28 in 3-D, 24 in 2-D), shared
                    // by the builder warps: warp b computes planes b, b + 8, ... of sample `lane`
                    unsigned char *slw = stage + (size_t)slot * kMmaSlotBytes;
                    const float *d0 = reinterpret_cast<const float *>(slw + kMmaStD0);
                    const int *rs = reinterpret_cast<const int *>(slw + kMmaStR);
                    constexpr int XT = D == 3 ? kMmaTX : 0;  // planes along N's grid dimension
#pragma unroll
                    for (int i = 0; i < (T::TAPS + NB - 1) / NB; ++i) {
                        const int jt = warp + NB * i;
                        if (jt >= T::TAPS) break;
                        const int reg = jt < XT ? 0 : (jt < XT + kMmaTY ? 1 : 2);  // x, y or z planes
                        const int t = jt - (reg == 0 ? 0 : (reg == 1 ? XT : XT + kMmaTY));
                        const int gd = D == 3 ? reg : reg - 1;  // grid dimension (2-D: y, z planes only)
                        const float d = d0[gd * B + lane] - (float)t;
                        // (a parameter array indexed at run time would be copied to local memory)
                        const float beta = gd == 0 ? g.beta2[0] : (gd == 1 ? g.beta2[1] : g.beta2[2]);
                        const float wv = ex2_approx(-beta * d * d);
                        const bool in = (unsigned)(t - rs[gd * B + lane]) < (unsigned)W;
                        reinterpret_cast<float *>(slw + (reg == 0 ? kMmaStWx : (reg == 1 ? kMmaStWy : kMmaStWz)))
                            [t * kMmaWS + lane] = in ? wv : 0.f;
                    }
                    asm volatile("bar.sync 1, %0;" ::"n"(NB * 32) : "memory");
                }
                // the MMAs of batch k - 2 (same operand buffer) have completed
                if (k >= 2 && !mbar_wait_bounded(&done[buf], (uint32_t)(((k >> 1) - 1) & 1)) && lane == 0)
                    atomicOr(status, kStatusSpreadTimeout);
                if constexpr (KAHAN) {
                    if (k >= 2) {
                        // batch k - 2's accumulator D[k % 2] into the group sum before batch k
                        // overwrites it
                        tc_fence_after();
                        mma_drain_batch_k2<CPW / 16>(tl, CPW * hk, kMmaColD + 64u * buf, k - 2);
                    }
                }
                const unsigned char *sl = stage + (size_t)slot * kMmaSlotBytes;
                // A: cells (y, z) of this lane, samples SPW hk .. SPW hk + SPW - 1
                const float4 *wy4 = reinterpret_cast<const float4 *>(sl + kMmaStWy) + (y * kMmaWS + SPW * hk) / 4;
                const float4 *wz4 = reinterpret_cast<const float4 *>(sl + kMmaStWz) + (z * kMmaWS + SPW * hk) / 4;
#pragma unroll
                for (int h = 0; h < SPW / 8; ++h) {  // 8 samples at a time: fewer live registers
                    float hi[8], lo[8];
#pragma unroll
                    for (int i = 0; i < 2; ++i) {
                        const float4 p = wy4[2 * h + i], s = wz4[2 * h + i];
                        float2 h0, l0, h1, l1;
                        tf32_split2(make_float2(p.x, p.y), make_float2(s.x, s.y), h0, l0);
                        tf32_split2(make_float2(p.z, p.w), make_float2(s.z, s.w), h1, l1);
                        hi[4 * i] = h0.x;
                        hi[4 * i + 1] = h0.y;
                        hi[4 * i + 2] = h1.x;
                        hi[4 * i + 3] = h1.y;
                        lo[4 * i] = l0.x;
                        lo[4 * i + 1] = l0.y;
                        lo[4 * i + 2] = l1.x;
                        lo[4 * i + 3] = l1.y;
                    }
                    tmem_st_x8(tl + 64u * buf + SPW * hk + 8u * h, hi);
                    tmem_st_x8(tl + 64u * buf + 32u + SPW * hk + 8u * h, lo);
                }
                const float2 *vs = reinterpret_cast<const float2 *>(sl + kMmaStV);
                unsigned char *bh = opB + (size_t)(2 * buf) * kBOp, *bl = bh + kBOp;
                if constexpr (D == 3) {
                    // B: rows (x = bx, coils bc0 .. bc0 + RPW / 2 - 1, re/im) for sample `lane`
                    const float wxk = reinterpret_cast<const float *>(sl + kMmaStWx)[bx * kMmaWS + lane];
#pragma unroll
                    for (int cc = 0; cc < RPW / 2; ++cc) {
                        const float2 vv = vs[(bc0 + cc) * B + lane];
                        const int nre = bx * 16 + (bc0 + cc) * 2;
                        float2 h, l;
                        tf32_split2(make_float2(wxk, wxk), vv, h, l);
                        *reinterpret_cast<float *>(bh + sw128_offset(nre, lane)) = h.x;
                        *reinterpret_cast<float *>(bl + sw128_offset(nre, lane)) = l.x;
                        *reinterpret_cast<float *>(bh + sw128_offset(nre + 1, lane)) = h.y;
                        *reinterpret_cast<float *>(bl + sw128_offset(nre + 1, lane)) = l.y;
                    }
                } else {
                    // B: rows (coil = warp, re/im) for sample `lane`: the coil value itself
                    const float2 vv = vs[warp * B + lane];
                    float2 h, l;
                    tf32_split2(make_float2(1.f, 1.f), vv, h, l);
                    *reinterpret_cast<float *>(bh + sw128_offset(2 * warp, lane)) = h.x;
                    *reinterpret_cast<float *>(bl + sw128_offset(2 * warp, lane)) = l.x;
                    *reinterpret_cast<float *>(bh + sw128_offset(2 * warp + 1, lane)) = h.y;
                    *reinterpret_cast<float *>(bl + sw128_offset(2 * warp + 1, lane)) = l.y;
                }
                mbar_arrive(&empty[slot]);
                if (!KAHAN && k % kMmaGroup == 0 && k > 0) {
                    // batch k starts a new group: once the previous group's MMAs are done,
                    // add its accumulator into S (the same phase is waited for again at
                    // k + 1, which returns at once)
                    if (!mbar_wait_bounded(&done[(k - 1) & 1], (uint32_t)(((k - 1) >> 1) & 1)) && lane == 0)
                        atomicOr(status, kStatusSpreadTimeout);
                    tc_fence_after();
                    mma_drain<N>(tl, hk, k == kMmaGroup);
                }
                // operands visible to the tensor core before the MMA warp proceeds
                tmem_wait_st();
                fence_proxy_async_smem();
                tc_fence_before();
                mbar_arrive(&ops[buf]);
            }

            // ---------------------------------------------------------------- epilogue
            if (nb > 0) {
                const int kl = nb - 1;
                if (!mbar_wait_bounded(&done[kl & 1], (uint32_t)((kl >> 1) & 1)) && lane == 0)
                    atomicOr(status, kStatusSpreadTimeout);
                tc_fence_after();
                if constexpr (KAHAN) {
                    // the last two batches' accumulators, in order
                    for (int j = max(0, nb - 2); j < nb; ++j) {
                        mma_drain_batch_k2<CPW / 16>(tl, CPW * hk, kMmaColD + 64u * (j & 1), j);
                        tmem_wait_st();  // G (and S, C) stored before the next drain reads them
                    }
                    // the last group's sum into S, C (S = G when there was one group)
                    mma_drain_kahan<CPW / 16>(tl, CPW * hk, kMmaColGK, nb <= kMmaGroup);
                    tmem_wait_st();
                }
            }
            // the unit's tile, read again here rather than kept in registers through the loop
            const int4 su = a.subs[unit / n_cg];
            int o[3], e[3];
            tile_coords<D>(g, su.x % g.ntiles, o, e);
            const int grp = su.x / g.ntiles;
            const bool split = (su.w & kSplitFlag) != 0;
            const bool inside = y < e[T::DY] && z < e[T::DZ];
            if constexpr (D == 3) {
                // this warp: lanes of quarter q, columns CPW hk .. (x planes CPW hk / 16 ..)
                const int64_t cell_yz = (int64_t)(o[1] + y) * g.nf[2] + (o[2] + z);
#pragma unroll
                for (int xi = 0; xi < CPW / 16; ++xi) {
                    // columns CPW hk + 16 xi ..: cell x = (CPW / 16) hk + xi, (coil, re/im) pairs
                    float dv[16];
                    if (nb > 0 && KAHAN) {
                        float cv[16];
                        tmem_ld_x16(tl + kMmaColSK + CPW * hk + 16u * xi, dv);
                        tmem_ld_x16(tl + kMmaColCK + CPW * hk + 16u * xi, cv);
                        tmem_wait_ld();
#pragma unroll
                        for (int i = 0; i < 16; ++i) dv[i] -= cv[i];
                    } else if (nb > 0) {
                        tmem_ld_x16(tl + kMmaColD + CPW * hk + 16u * xi, dv);
                        if (nb > kMmaGroup) {  // plus the drained groups
                            float sv[16];
                            tmem_ld_x16(tl + kMmaColD + N + CPW * hk + 16u * xi, sv);
                            tmem_wait_ld();
#pragma unroll
                            for (int i = 0; i < 16; ++i) dv[i] += sv[i];
                        } else {
                            tmem_wait_ld();
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < 16; ++i) dv[i] = 0.f;
                    }
                    const int x = (CPW / 16) * hk + xi;
                    if (!inside || x >= e[0]) continue;
                    const int64_t cell = (int64_t)(o[0] + x) * g.nf[1] * g.nf[2] + cell_yz;
#pragma unroll
                    for (int c = 0; c < CG; ++c) {
                        if (cg0 + c >= g.n_coil) break;
                        float2 *dst = a.grid + ((int64_t)grp * g.n_coil + cg0 + c) * g.G + cell;
                        if (split) {
                            atomicAdd(&dst->x, dv[2 * c]);
                            atomicAdd(&dst->y, dv[2 * c + 1]);
                        } else {
                            *dst = make_float2(dv[2 * c], dv[2 * c + 1]);
                        }
                    }
                }
            } else {
                // this warp: lanes of quarter q, columns 8 hk .. 8 hk + 7 (coils 4 hk .. 4 hk + 3)
                float dv[8];
                if (nb > 0) {
                    tmem_ld_x8(tl + kMmaColD + 8u * hk, dv);
                    if (nb > kMmaGroup) {  // plus the drained groups
                        float sv[8];
                        tmem_ld_x8(tl + kMmaColD + N + 8u * hk, sv);
                        tmem_wait_ld();
#pragma unroll
                        for (int i = 0; i < 8; ++i) dv[i] += sv[i];
                    } else {
                        tmem_wait_ld();
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 8; ++i) dv[i] = 0.f;
                }
                if (inside) {
                    const int64_t cell = (int64_t)(o[0] + y) * g.nf[1] + (o[1] + z);
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) {
                        const int c = 4 * hk + cc;
                        if (cg0 + c >= g.n_coil) break;
                        float2 *dst = a.grid + ((int64_t)grp * g.n_coil + cg0 + c) * g.G + cell;
                        if (split) {
                            atomicAdd(&dst->x, dv[2 * cc]);
                            atomicAdd(&dst->y, dv[2 * cc + 1]);
                        } else {
                            *dst = make_float2(dv[2 * cc], dv[2 * cc + 1]);
                        }
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == WM) tmem_dealloc(tbase, kCols);
}


}  // namespace gbn
