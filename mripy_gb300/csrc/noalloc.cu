// gbn_spread2d_noalloc: the 2-D spread (gridding stage of the type-1 transform) without any
// device allocation.
//
// Some callers cannot allocate device memory where they need the gridding: code running
// inside a host framework that owns the GPU's memory pool and forbids side allocations,
// real-time reconstruction loops that must never block in cudaMalloc, and plugin hosts that
// hand a library only pre-sized input and output buffers.  This entry point serves them.  The
// caller passes the coordinates, the samples and the output grid; every other buffer the
// binning needs (packed sample records, per-tile counts and offsets, the (sample, tile)
// list and the work table) lives in one file-scope __device__ array of fixed size, so no
// cudaMalloc, cudaFree or allocating library routine is called.
//
// Limits: at most GBN_NOALLOC_MAX_SAMPLES samples and GBN_NOALLOC_MAX_TILES output tiles
// (16 x 32 grid cells each) per call, at most 16 taps per dimension (nspread <= 8), and an
// oversampled grid made of whole tiles (ms a multiple of 8, mt of 16) at least one tile plus
// one stencil wide; anything else is rejected with GBN_ERR_CAPACITY before any work is
// queued.  The array (about 8.7 MiB) is held by every GPU that loads the library until the
// process exits.
//
// Sharing: every call reuses the same array and overwrites what the last call left there
// (the per-tile counters are cleared at the start of each call).  Calls whose work overlaps
// on the GPU -- issued on different streams, or from different host threads without ordering
// -- race on the array and corrupt each other's results: order them on one stream.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current (host code must not pass the symbol
// itself: on the host it is only a stand-in, not a device address), and keeps it for the
// life of the process.  Under CUDA's lazy module loading that first call is also where the
// driver commits the array's memory on the device, so it can fail for lack of memory: make
// it during set-up, before any stream capture.  The kept address belongs to the device's
// primary context (the runtime's); after cudaDeviceReset, or from another driver context
// on the same device, it is stale, so such callers must not use this entry point.
//
// Non-finite coordinates are not reported here (that would need a host synchronisation);
// a sample with a non-finite coordinate is left out: it reaches no tile and adds nothing
// to the grid.  The result matches gbn_spread on the same (finite) inputs up to FP32
// summation order.
#include <cmath>
#include <mutex>
#include <string>

#include "common.cuh"
#include "grid2d_kernels.cuh"

namespace gbn {
namespace {

constexpr int kNaTX = 16, kNaTY = 32;   // output tile (cells)
constexpr int kNaMaxSub = 256;          // samples per work item
constexpr int kNaTouch = 4;             // tiles one stencil reaches at most (tile >= stencil)
constexpr int kNaThreads = 256;

constexpr size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
constexpr size_t kMaxEntries = (size_t)kNaTouch * GBN_NOALLOC_MAX_SAMPLES;
constexpr size_t kMaxSubs = GBN_NOALLOC_MAX_TILES + kMaxEntries / kNaMaxSub;
// layout of the scratch array (byte offsets)
constexpr size_t kOffPts = 0;
constexpr size_t kOffIdx = align256(kOffPts + sizeof(float4) * GBN_NOALLOC_MAX_SAMPLES);
constexpr size_t kOffCount = align256(kOffIdx + sizeof(uint32_t) * kMaxEntries);
constexpr size_t kOffCursor = align256(kOffCount + sizeof(uint32_t) * GBN_NOALLOC_MAX_TILES);
constexpr size_t kOffTileOff = align256(kOffCursor + sizeof(uint32_t) * GBN_NOALLOC_MAX_TILES);
constexpr size_t kOffSubOff = align256(kOffTileOff + sizeof(uint32_t) * GBN_NOALLOC_MAX_TILES);
constexpr size_t kOffSubs = align256(kOffSubOff + sizeof(uint32_t) * GBN_NOALLOC_MAX_TILES);
constexpr size_t kOffMeta = align256(kOffSubs + sizeof(int4) * kMaxSubs);
constexpr size_t kScratchBytes = align256(kOffMeta + 256);

}  // namespace
}  // namespace gbn

// The one scratch array of gbn_spread2d_noalloc (see the file comment).
static __device__ __align__(256) unsigned char g_noalloc_scratch[gbn::kScratchBytes];

namespace gbn {
namespace {

constexpr double kTwoPiNa = 6.283185307179586476925286766559;

__device__ inline double na_py_mod(double a, double b) {
    double m = fmod(a, b);
    if (m != 0.0) {
        if ((b < 0) != (m < 0)) m += b;
    } else {
        m = copysign(0.0, b);
    }
    return m;
}
__device__ inline double na_py_floordiv(double a, double b) {
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

struct NaGeom {
    int M, ns, W, nf0, nf1, nt0, nt1, ntiles, n_coil;
    float beta0, beta1;
    double df;
};

// per sample: packed record (same format as the plan's) and the per-tile counts.  A sample
// with a non-finite coordinate gets the record's z slot set to 1 (unused in 2-D, else 0)
// and is counted in no tile, so the scatter lists it nowhere and the spread never reads it.
template <typename T>
__global__ void k_na_prep(const T *__restrict__ x, const T *__restrict__ y, NaGeom g, float4 *__restrict__ pts,
                          uint32_t *__restrict__ count) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.M) return;
    const T *src[2] = {x, y};
    const int nf[2] = {g.nf0, g.nf1};
    float f[2] = {0.f, 0.f};
    int c0[2] = {0, 0};
    for (int d = 0; d < 2; ++d) {
        const double xs = (double)src[d][j] * g.df;
        if (!isfinite(xs)) {
            pts[j] = make_float4(0.f, 0.f, 1.f, 0.f);
            return;
        }
        const double h = kTwoPiNa / nf[d];
        const double xi = na_py_mod(xs, kTwoPiNa);
        const int64_t m = 1 + (int64_t)na_py_floordiv(xi, h);
        f[d] = (float)((xi - h * (double)(m - 1)) / h);
        int64_t first = (m - g.ns) % nf[d];
        c0[d] = (int)(first < 0 ? first + nf[d] : first);
    }
    pts[j] = make_float4(f[0], f[1], 0.f, __uint_as_float(pack_cells(2, c0[0], c0[1], 0)));
    const int n0 = touched_tiles(c0[0], g.W, g.nf0, kNaTX, g.nt0);
    const int n1 = touched_tiles(c0[1], g.W, g.nf1, kNaTY, g.nt1);
    for (int a = 0; a < n0; ++a)
        for (int b = 0; b < n1; ++b)
            atomicAdd(&count[((c0[0] / kNaTX + a) % g.nt0) * g.nt1 + (c0[1] / kNaTY + b) % g.nt1], 1u);
}

// exclusive scan of n <= GBN_NOALLOC_MAX_TILES values by one block of 1024 threads
__device__ void na_block_scan(const uint32_t *in, uint32_t *out, int n, uint32_t *total, uint32_t (*xform)(uint32_t)) {
    __shared__ uint32_t warp_tot[32];
    constexpr int kChunk = GBN_NOALLOC_MAX_TILES / 1024;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t local[kChunk];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kChunk; ++k) {
        const int i = t * kChunk + k;
        local[k] = i < n ? xform(in[i]) : 0u;
        sum += local[k];
    }
    uint32_t v = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += u;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_tot[lane];
        uint32_t wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, wi, off);
            if (lane >= off) wi += u;
        }
        warp_tot[lane] = wi - w;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    uint32_t run = v - sum + warp_tot[warp];
#pragma unroll
    for (int k = 0; k < kChunk; ++k) {
        const int i = t * kChunk + k;
        if (i < n) out[i] = run;
        run += local[k];
    }
    __syncthreads();
}

__device__ uint32_t na_identity(uint32_t v) { return v; }
__device__ uint32_t na_nsub(uint32_t v) { return v == 0 ? 1u : (v + kNaMaxSub - 1) / kNaMaxSub; }

// tile offsets, cleared cursors and the work table; meta[0] = number of work items.
// One block of 1024 threads does it all: each thread scans up to 16 tile counts, and the
// thread of a tile writes that tile's work items one by one (up to M / 256 for a tile that
// holds every sample).  Serial work, but small next to the spread, and it needs no second
// launch or grid-wide synchronisation.
__global__ void __launch_bounds__(1024) k_na_layout(int ntiles, uint32_t *__restrict__ count,
                                                    uint32_t *__restrict__ tile_off, uint32_t *__restrict__ sub_off,
                                                    uint32_t *__restrict__ cursor, int4 *__restrict__ subs,
                                                    uint32_t *__restrict__ meta) {
    __shared__ uint32_t tot[2];
    na_block_scan(count, tile_off, ntiles, &tot[0], na_identity);
    na_block_scan(count, sub_off, ntiles, &tot[1], na_nsub);
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
        cursor[t] = 0u;
        const uint32_t c = count[t];
        const uint32_t s = na_nsub(c);
        for (uint32_t k = 0; k < s; ++k) {
            const uint32_t start = k * kNaMaxSub;
            const uint32_t len = c > start ? min((uint32_t)kNaMaxSub, c - start) : 0u;
            const int flags = (s > 1 ? kSplitFlag : 0) | (k == 0 ? kFirstFlag : 0);
            subs[sub_off[t] + k] = make_int4(t, (int)(tile_off[t] + start), (int)len, flags);
        }
    }
    if (threadIdx.x == 0) meta[0] = tot[1];
}

__global__ void k_na_scatter(NaGeom g, const float4 *__restrict__ pts, const uint32_t *__restrict__ tile_off,
                             uint32_t *__restrict__ cursor, uint32_t *__restrict__ idx) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.M) return;
    const float4 p = pts[j];
    if (p.z != 0.f) return;  // non-finite coordinate: in no tile
    int c0x, c0y, c0z;
    unpack_cells(2, __float_as_uint(p.w), c0x, c0y, c0z);
    const int n0 = touched_tiles(c0x, g.W, g.nf0, kNaTX, g.nt0);
    const int n1 = touched_tiles(c0y, g.W, g.nf1, kNaTY, g.nt1);
    for (int a = 0; a < n0; ++a)
        for (int b = 0; b < n1; ++b) {
            const int t = ((c0x / kNaTX + a) % g.nt0) * g.nt1 + (c0y / kNaTY + b) % g.nt1;
            idx[tile_off[t] + atomicAdd(&cursor[t], 1u)] = (uint32_t)j;
        }
}

__global__ void k_na_zero(NaGeom g, const int4 *__restrict__ subs, const uint32_t *__restrict__ meta,
                          float2 *__restrict__ grid) {
    if (blockIdx.x >= meta[0]) return;
    const int4 sub = subs[blockIdx.x];
    if (!((sub.w & kSplitFlag) && (sub.w & kFirstFlag))) return;
    const int o0 = (sub.x / g.nt1) * kNaTX, o1 = (sub.x % g.nt1) * kNaTY;
    const int e0 = min(kNaTX, g.nf0 - o0), e1 = min(kNaTY, g.nf1 - o1);
    const int64_t G = (int64_t)g.nf0 * g.nf1;
    for (int coil = 0; coil < g.n_coil; ++coil)
        for (int i = threadIdx.x; i < e0 * e1; i += blockDim.x)
            grid[coil * G + (int64_t)(o0 + i / e1) * g.nf1 + o1 + i % e1] = make_float2(0.f, 0.f);
}

constexpr int kNaBatch = 64;

// the warp-owned-row spread of k_spread2d, reading each sample record through the list
template <int CG>
__global__ void __launch_bounds__(kNaThreads) k_na_spread(NaGeom g, const int4 *__restrict__ subs,
                                                          const uint32_t *__restrict__ meta,
                                                          const float4 *__restrict__ pts,
                                                          const uint32_t *__restrict__ idx,
                                                          const float2 *__restrict__ c, int64_t c_elem,
                                                          int64_t c_coil, float2 *__restrict__ grid) {
    using L = Lanes2D<0, CG>;
    __shared__ float2 acc[kNaTX * kNaTY * CG];
    __shared__ float st_w[kNaBatch * 32];
    __shared__ float2 st_v[kNaBatch * CG];
    __shared__ int2 st_r[kNaBatch];
    if (blockIdx.x >= meta[0]) return;
    const int4 sub = subs[blockIdx.x];
    const int cg0 = blockIdx.y * CG;
    const int o0 = (sub.x / g.nt1) * kNaTX, o1 = (sub.x % g.nt1) * kNaTY;
    const int e0 = min(kNaTX, g.nf0 - o0), e1 = min(kNaTY, g.nf1 - o1);
    const int W = g.W, ns = g.ns, nf0 = g.nf0, nf1 = g.nf1;
    for (int i = threadIdx.x; i < kNaTX * kNaTY * CG; i += blockDim.x) acc[i] = make_float2(0.f, 0.f);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int cl = lane % CG, q = lane / CG;
    const int R = (kNaTX + nw - 1) / nw;
    const int row0 = warp * R, row1 = min(row0 + R, e0);
    for (int base = 0; base < sub.z; base += kNaBatch) {
        const int n = min(kNaBatch, sub.z - base);
        __syncthreads();
        for (int i = threadIdx.x; i < n * 32; i += blockDim.x) {
            const int s = i >> 5, k = i & 31, kq = k & 15;
            const float4 p = pts[idx[sub.y + base + s]];
            float val = 0.f;
            if (kq < W) {
                const float d = (k < 16 ? p.x : p.y) + (float)(ns - 1 - kq);
                val = exp2f(-(k < 16 ? g.beta0 : g.beta1) * d * d);
            }
            st_w[i] = val;
            if (k == 0) {
                int c0x, c0y, c0z;
                unpack_cells(2, __float_as_uint(p.w), c0x, c0y, c0z);
                int rx = c0x - o0, ry = c0y - o1;
                rx += rx < 0 ? nf0 : 0;
                ry += ry < 0 ? nf1 : 0;
                rx -= rx > nf0 - W ? nf0 : 0;
                ry -= ry > nf1 - W ? nf1 : 0;
                st_r[s] = make_int2(rx, ry);
            }
        }
        for (int i = threadIdx.x; i < n * CG; i += blockDim.x) {
            const int s = i / CG, cc = i - s * CG;
            const uint32_t j = idx[sub.y + base + s];
            st_v[i] = cg0 + cc < g.n_coil ? c[(int64_t)j * c_elem + (int64_t)(cg0 + cc) * c_coil]
                                          : make_float2(0.f, 0.f);
        }
        __syncthreads();
        for (int s = 0; s < n; ++s) {
            const int2 r = st_r[s];
            const int lo = max(row0, r.x), hi = min(row1, r.x + W);
            if (lo >= hi) continue;
            const float2 v = st_v[s * CG + cl];
            const float *w = st_w + s * 32;
            float wy[L::KT];
            int ly[L::KT];
#pragma unroll
            for (int t = 0; t < L::KT; ++t) {
                const int ky = q + t * L::NQ;
                const int yy = r.y + ky;
                const bool ok = ky < W && (unsigned)yy < (unsigned)e1;
                wy[t] = ok ? w[16 + ky] : 0.f;
                ly[t] = ok ? yy : -1;
            }
            for (int row = lo; row < hi; ++row) {
                const float wx = w[row - r.x];
                float2 *dst = acc + (size_t)row * kNaTY * CG + cl;
#pragma unroll
                for (int t = 0; t < L::KT; ++t) {
                    if (ly[t] >= 0) {
                        float2 *cell = dst + (size_t)ly[t] * CG;
                        const float ww = wx * wy[t];
                        float2 o = *cell;
                        o.x = fmaf(ww, v.x, o.x);
                        o.y = fmaf(ww, v.y, o.y);
                        *cell = o;
                    }
                }
            }
        }
    }
    __syncthreads();
    const bool split = (sub.w & kSplitFlag) != 0;
    const int64_t G = (int64_t)nf0 * nf1;
    for (int i = threadIdx.x; i < e0 * e1 * CG; i += blockDim.x) {
        const int cc = i % CG, cell = i / CG;
        if (cg0 + cc >= g.n_coil) continue;
        const int lx = cell / e1, lyy = cell - lx * e1;
        const float2 val = acc[((size_t)lx * kNaTY + lyy) * CG + cc];
        float2 *dst = grid + (int64_t)(cg0 + cc) * G + (int64_t)(o0 + lx) * nf1 + (o1 + lyy);
        if (split) {
            atomicAdd(&dst->x, val.x);
            atomicAdd(&dst->y, val.y);
        } else {
            *dst = val;
        }
    }
}

// device address of the scratch array, looked up once per device
std::mutex g_na_mutex;
void *g_na_ptr[64] = {};

int na_scratch(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return record_error(GBN_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return record_error(GBN_ERR_CAPACITY, "device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return record_error(GBN_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
        g_na_ptr[dev] = p;
    }
    *out = (unsigned char *)g_na_ptr[dev];
    return GBN_OK;
}

}  // namespace
}  // namespace gbn

using namespace gbn;

extern "C" int gbn_spread2d_noalloc(int coord_dtype, const void *x, const void *y, int64_t M, const void *c,
                                    gbn_layout c_layout, int32_t n_coil, int32_t ms, int32_t mt, double eps,
                                    double df, void *grid, gbn_stream_t stream) {
    if (coord_dtype != GBN_COORD_F32 && coord_dtype != GBN_COORD_F64)
        return record_error(GBN_ERR_ARG, "bad coordinate dtype");
    if (M < 0 || n_coil < 1 || !grid || !std::isfinite(df)) return record_error(GBN_ERR_ARG, "bad argument");
    if (M > 0 && (!x || !y || !c)) return record_error(GBN_ERR_ARG, "null buffer");
    if (M > GBN_NOALLOC_MAX_SAMPLES)
        return record_error(GBN_ERR_CAPACITY, "gbn_spread2d_noalloc takes at most GBN_NOALLOC_MAX_SAMPLES "
                                              "(262144) samples per call; use gbn_spread with a plan");
    int ns = 0;
    int64_t nf[3];
    double tau = 0;
    int st = gbn_grid_params(2, ms, mt, 1, eps, 0, &ns, nf, &tau);
    if (st != GBN_OK) return st;
    const int W = 2 * ns;
    if (W > 16) return record_error(GBN_ERR_CAPACITY, "gbn_spread2d_noalloc supports nspread <= 8 (eps >= ~2e-8)");
    // whole tiles only: then a stencil of <= 16 taps reaches at most 2 x 2 tiles, which bounds
    // the (sample, tile) list at 4 entries per sample
    if (nf[0] < kNaTX + W || nf[1] < kNaTY + W || nf[0] % kNaTX != 0 || nf[1] % kNaTY != 0)
        return record_error(GBN_ERR_CAPACITY, "gbn_spread2d_noalloc needs an oversampled grid of whole 16x32 tiles "
                                              "at least one tile plus the stencil wide (ms % 8 == 0, mt % 16 == 0)");
    NaGeom g;
    g.M = (int)M;
    g.ns = ns;
    g.W = W;
    g.nf0 = (int)nf[0];
    g.nf1 = (int)nf[1];
    g.nt0 = (g.nf0 + kNaTX - 1) / kNaTX;
    g.nt1 = (g.nf1 + kNaTY - 1) / kNaTY;
    g.ntiles = g.nt0 * g.nt1;
    g.n_coil = n_coil;
    g.df = df;
    const double h0 = 6.283185307179586 / g.nf0, h1 = 6.283185307179586 / g.nf1;
    g.beta0 = (float)(h0 * h0 / (4.0 * tau) * 1.4426950408889634);
    g.beta1 = (float)(h1 * h1 / (4.0 * tau) * 1.4426950408889634);
    if (g.ntiles > GBN_NOALLOC_MAX_TILES)
        return record_error(GBN_ERR_CAPACITY, "oversampled grid needs more than GBN_NOALLOC_MAX_TILES (16384) tiles");

    unsigned char *base = nullptr;
    st = na_scratch(&base);
    if (st != GBN_OK) return st;
    float4 *pts = (float4 *)(base + kOffPts);
    uint32_t *idx = (uint32_t *)(base + kOffIdx);
    uint32_t *count = (uint32_t *)(base + kOffCount);
    uint32_t *cursor = (uint32_t *)(base + kOffCursor);
    uint32_t *tile_off = (uint32_t *)(base + kOffTileOff);
    uint32_t *sub_off = (uint32_t *)(base + kOffSubOff);
    int4 *subs = (int4 *)(base + kOffSubs);
    uint32_t *meta = (uint32_t *)(base + kOffMeta);
    cudaStream_t s = (cudaStream_t)stream;

    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(uint32_t) * g.ntiles, s);
    if (e == cudaSuccess && M > 0) {
        const unsigned blocks = (unsigned)((M + 255) / 256);
        if (coord_dtype == GBN_COORD_F64)
            k_na_prep<double><<<blocks, 256, 0, s>>>((const double *)x, (const double *)y, g, pts, count);
        else
            k_na_prep<float><<<blocks, 256, 0, s>>>((const float *)x, (const float *)y, g, pts, count);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_na_layout<<<1, 1024, 0, s>>>(g.ntiles, count, tile_off, sub_off, cursor, subs, meta);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && M > 0) {
        k_na_scatter<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(g, pts, tile_off, cursor, idx);
        e = cudaGetLastError();
    }
    // upper bound of the work items; blocks beyond meta[0] return at once
    const int64_t bound = (int64_t)g.ntiles + ((int64_t)kNaTouch * M + kNaMaxSub - 1) / kNaMaxSub;
    if (e == cudaSuccess) {
        k_na_zero<<<(unsigned)bound, 256, 0, s>>>(g, subs, meta, (float2 *)grid);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        int cg = 8;
        while (cg > 1 && cg > n_coil) cg /= 2;
        const dim3 blocks((unsigned)bound, (unsigned)((n_coil + cg - 1) / cg));
        const float2 *cc = (const float2 *)c;
        switch (cg) {
            case 8: k_na_spread<8><<<blocks, kNaThreads, 0, s>>>(g, subs, meta, pts, idx, cc, c_layout.elem_stride,
                                                                  c_layout.coil_stride, (float2 *)grid); break;
            case 4: k_na_spread<4><<<blocks, kNaThreads, 0, s>>>(g, subs, meta, pts, idx, cc, c_layout.elem_stride,
                                                                  c_layout.coil_stride, (float2 *)grid); break;
            case 2: k_na_spread<2><<<blocks, kNaThreads, 0, s>>>(g, subs, meta, pts, idx, cc, c_layout.elem_stride,
                                                                  c_layout.coil_stride, (float2 *)grid); break;
            default: k_na_spread<1><<<blocks, kNaThreads, 0, s>>>(g, subs, meta, pts, idx, cc, c_layout.elem_stride,
                                                                   c_layout.coil_stride, (float2 *)grid); break;
        }
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return record_error(GBN_ERR_CUDA, cudaGetErrorString(e));
    return GBN_OK;
}
