// Deapodisation fused with the oversampling pad (before the forward FFT) and the
// crop (after the inverse FFT), plus the SENSE-fused variants.
//
// The reference multiplies by (pi/tau)^(d/2) exp(tau |k|^2) on the host and then
// zero-pads / crops with numpy slicing (fft/nufft_func.py:751-764, 728-738).  Here the
// separable factor is a per-dimension table built in FP64 on the GPU,
//     tab_d[i] = sqrt(pi/tau) exp(tau k^2) / nf_d,   k = i - m_d/2,
// so the product over d also carries the 1/N of the reference's interp (type-2) and of
// its normalised inverse FFT (type-1).  The pad writes every grid cell (zeros outside
// the image band), so no separate memset precedes the FFT.
//
// Work decomposition.  Images are (group, pixel, coil) with arbitrary strides, usually
// coil-last; grids are coil-major (instance = group * n_coil + coil, then nf_0 .. nf_{D-1}).
// Both pad and crop are therefore transposes, done through shared memory by "band"
// blocks: a band block owns one image row (group, outer pixel index) or a segment of it,
// for a chunk of coils.  It reads the pixels of all its coils in the image's own order
// (coalesced whether coil-last or coil-major), scales them by the tables, and writes
// whole grid rows (pad) or reads the two band runs of each grid row (crop).
// The rest of the padded grid is two kinds of contiguous zero slabs per instance:
// the out-of-band x planes (dim >= 2) and, in 3-D, the out-of-band y rows of each in-band
// x plane.  "Zero" blocks of the same launch fill them in fixed chunks with 16-byte stores.
#include <algorithm>

#include "common.cuh"

namespace gbn {

namespace {

constexpr int kStageElems = 4096;  // staged complex values per band block (32 KB)
constexpr int64_t kMinBandBlocks = 1024;  // band blocks a pad/crop launch aims for (~7 per SM)
constexpr int kZeroChunk = 8192;   // cells per zero block
constexpr int kThreads = 256;
constexpr int kSenseSeg = 1024;    // crop_sense: at most 4 pixels per thread

__global__ void k_build_table(int m, int nf, double tau, float *tab) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const double pi = 3.14159265358979323846;
    double k = (double)(i - m / 2);
    tab[i] = (float)(sqrt(pi / tau) * exp(tau * k * k) / (double)nf);
}

__global__ void k_fill_one(float *tab) { tab[0] = 1.f; }

// entry D - 1 of a kernel argument's per-axis array, read with constant indices (a run-time
// index would copy the whole argument block to local memory in every thread)
template <class T>
__device__ __forceinline__ T last_axis(const T (&v)[3], int D) {
    return D == 3 ? v[2] : (D == 2 ? v[1] : v[0]);
}

// grid index of image index i along one dim: band cells are [0, m - m/2) and [nf - m/2, nf)
__device__ __forceinline__ int grid_index(int i, int m, int nf) {
    const int g = i - m / 2;
    return g < 0 ? g + nf : g;
}

struct Decomp {
    int64_t n_outer;          // image rows per group: prod_{d < D-1} m_d
    int seg, nseg;            // segment of the last image dim per band block, segments per row
    int cc, ncc;              // coils per chunk, chunks (crop_sense: chunks looped in-block)
    int64_t nband;            // band blocks
    int64_t x_len, x_chunks;  // out-of-band x slab of an instance (dim >= 2)
    int64_t y_len, y_chunks;  // dim 3: out-of-band y slab of one in-band x plane
    int64_t nzero;            // zero blocks
    bool coil_fast;           // image coil stride below its pixel stride: stage coils fastest
};

// The band block's row: group, outer pixel prefix, table product and grid row prefix.
struct BandRow {
    int64_t grp, p, gbase;
    int i0, seg_len, c0, n_cc, seg_i;
    float s;
};

__device__ __forceinline__ BandRow band_row(const DeapodArgs &a, const Decomp &dc, int64_t b, bool chunked) {
    const Geom &g = a.g;
    const int D = g.dim;
    BandRow r;
    r.seg_i = (int)(b % dc.nseg);
    b /= dc.nseg;
    int chunk = 0;
    if (chunked) {
        chunk = (int)(b % dc.ncc);
        b /= dc.ncc;
    }
    r.p = b % dc.n_outer;
    r.grp = b / dc.n_outer;
    r.s = 1.f;
    r.gbase = 0;
    if (D == 3) {
        const int i0 = (int)(r.p / a.m[1]), i1 = (int)(r.p - (int64_t)i0 * a.m[1]);
        r.s = a.tab[0][i0] * a.tab[1][i1];
        r.gbase = (int64_t)grid_index(i0, a.m[0], g.nf[0]) * g.nf[1] + grid_index(i1, a.m[1], g.nf[1]);
    } else if (D == 2) {
        r.s = a.tab[0][r.p];
        r.gbase = grid_index((int)r.p, a.m[0], g.nf[0]);
    }
    const int ml = last_axis(a.m, D);
    r.i0 = r.seg_i * dc.seg;
    r.seg_len = min(dc.seg, ml - r.i0);
    r.c0 = chunk * dc.cc;
    r.n_cc = min(dc.cc, g.n_coil - r.c0);
    return r;
}

// zero cells [start, end) of the grid: 16-byte stores between a scalar head and tail
__device__ __forceinline__ void zero_range(float2 *grid, int64_t start, int64_t end) {
    float2 *p = grid + start;
    int64_t n = end - start;
    if (n <= 0) return;
    if (reinterpret_cast<uintptr_t>(p) & 15) {
        if (threadIdx.x == 0) *p = make_float2(0.f, 0.f);
        ++p;
        --n;
    }
    float4 *q = reinterpret_cast<float4 *>(p);
    const int64_t n4 = n >> 1;
    for (int64_t i = threadIdx.x; i < n4; i += blockDim.x) q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if ((n & 1) && threadIdx.x == 0) p[n - 1] = make_float2(0.f, 0.f);
}

__device__ __forceinline__ void zero_block(const DeapodArgs &a, const Decomp &dc, int64_t z, float2 *grid) {
    const Geom &g = a.g;
    const int64_t n_inst = (int64_t)g.n_coil * g.n_traj;
    int64_t start, end;
    if (z < n_inst * dc.x_chunks) {
        const int64_t inst = z / dc.x_chunks, ch = z - inst * dc.x_chunks;
        const int64_t s0 = inst * g.G + (int64_t)(a.m[0] - a.m[0] / 2) * (g.G / g.nf[0]);
        start = s0 + ch * kZeroChunk;
        end = min(s0 + dc.x_len, start + (int64_t)kZeroChunk);
    } else {
        z -= n_inst * dc.x_chunks;
        const int64_t slab = z / dc.y_chunks, ch = z - slab * dc.y_chunks;
        const int64_t inst = slab / a.m[0];
        const int ix = (int)(slab - inst * a.m[0]);
        const int64_t s0 = inst * g.G +
                           ((int64_t)grid_index(ix, a.m[0], g.nf[0]) * g.nf[1] + (a.m[1] - a.m[1] / 2)) * g.nf[2];
        start = s0 + ch * kZeroChunk;
        end = min(s0 + dc.y_len, start + (int64_t)kZeroChunk);
    }
    zero_range(grid, start, end);
}

// Pad sources: the scaled pixel value of (group, pixel, coil).
struct ImageSrc {
    const float2 *img;
    gbn_layout L;
    __device__ __forceinline__ float2 operator()(int64_t grp, int64_t pix, int coil) const {
        return img[grp * L.traj_stride + pix * L.elem_stride + (int64_t)coil * L.coil_stride];
    }
};

struct SenseSrc {  // x[grp] * sens[coil]
    const float2 *x;
    gbn_layout XL;
    const float2 *sens;
    gbn_layout SL;
    __device__ __forceinline__ float2 operator()(int64_t grp, int64_t pix, int coil) const {
        const float2 v = x[grp * XL.traj_stride + pix * XL.elem_stride];
        const float2 s = sens[pix * SL.elem_stride + (int64_t)coil * SL.coil_stride];
        return make_float2(v.x * s.x - v.y * s.y, v.x * s.y + v.y * s.x);
    }
};

template <class Src>
__global__ void __launch_bounds__(kThreads) k_pad(DeapodArgs a, Decomp dc, Src src, float2 *__restrict__ grid) {
    extern __shared__ float2 st_pad[];
    if (blockIdx.x >= dc.nband) {
        zero_block(a, dc, (int64_t)blockIdx.x - dc.nband, grid);
        return;
    }
    const Geom &g = a.g;
    const int D = g.dim;
    const int ml = last_axis(a.m, D), Ld = last_axis(g.nf, D);
    const float *tl = last_axis(a.tab, D);
    const BandRow r = band_row(a, dc, blockIdx.x, true);
    const int SP = dc.seg + 1;

    // stage the scaled pixels of the segment for the coil chunk (unrolled: several image
    // loads in flight per thread)
    const int n = r.n_cc * r.seg_len;
#pragma unroll 4
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
        int cc, k;
        if (dc.coil_fast) {
            k = idx / r.n_cc;
            cc = idx - k * r.n_cc;
        } else {
            cc = idx / r.seg_len;
            k = idx - cc * r.seg_len;
        }
        const int i = r.i0 + k;
        const float2 v = src(r.grp, r.p * ml + i, r.c0 + cc);
        const float f = r.s * tl[i];
        st_pad[cc * SP + k] = make_float2(v.x * f, v.y * f);
    }
    __syncthreads();

    // write the grid rows: the segment's band cells, then its share of the zero middle
    const int Zm = Ld - ml;
    const int z0 = (int)((int64_t)Zm * r.seg_i / dc.nseg), z1 = (int)((int64_t)Zm * (r.seg_i + 1) / dc.nseg);
    const int len = r.seg_len + (z1 - z0);
    const int nch = (len + 31) >> 5;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int w = warp; w < r.n_cc * nch; w += nw) {
        const int cc = w / nch;
        const int k = (w - cc * nch) * 32 + lane;
        if (k >= len) continue;
        float2 *row = grid + (r.grp * g.n_coil + r.c0 + cc) * g.G + r.gbase * Ld;
        if (k < r.seg_len) {
            row[grid_index(r.i0 + k, ml, Ld)] = st_pad[cc * SP + k];
        } else {
            row[(ml - ml / 2) + z0 + (k - r.seg_len)] = make_float2(0.f, 0.f);
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_crop(DeapodArgs a, Decomp dc, const float2 *__restrict__ grid,
                                                   float2 *__restrict__ img, gbn_layout L) {
    extern __shared__ float2 st_crop[];
    const Geom &g = a.g;
    const int D = g.dim;
    const int ml = last_axis(a.m, D), Ld = last_axis(g.nf, D);
    const float *tl = last_axis(a.tab, D);
    const BandRow r = band_row(a, dc, blockIdx.x, true);
    const int SP = dc.seg + 1;
    const float s = a.grp_scale ? r.s * a.grp_scale[r.grp] : r.s;

    // read the band runs of the coil chunk's grid rows (unrolled: several grid loads in
    // flight per warp)
    const int nch = (r.seg_len + 31) >> 5;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll 4
    for (int w = warp; w < r.n_cc * nch; w += nw) {
        const int cc = w / nch;
        const int k = (w - cc * nch) * 32 + lane;
        if (k >= r.seg_len) continue;
        const int i = r.i0 + k;
        const float2 v = grid[(r.grp * g.n_coil + r.c0 + cc) * g.G + r.gbase * Ld + grid_index(i, ml, Ld)];
        const float f = s * tl[i];
        st_crop[cc * SP + k] = make_float2(v.x * f, v.y * f);
    }
    __syncthreads();

    // write the image pixels in the image's own order
    const int n = r.n_cc * r.seg_len;
    float2 *dst = img + r.grp * L.traj_stride;
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
        int cc, k;
        if (dc.coil_fast) {
            k = idx / r.n_cc;
            cc = idx - k * r.n_cc;
        } else {
            cc = idx / r.seg_len;
            k = idx - cc * r.seg_len;
        }
        dst[(r.p * ml + r.i0 + k) * L.elem_stride + (int64_t)(r.c0 + cc) * L.coil_stride] = st_crop[cc * SP + k];
    }
}

// x[grp] = sum_coil conj(sens[coil]) * crop(deapod * grid[(grp, coil)])
__global__ void __launch_bounds__(kThreads) k_crop_sense(DeapodArgs a, Decomp dc, const float2 *__restrict__ grid,
                                                         const float2 *__restrict__ sens, gbn_layout SL,
                                                         float2 *__restrict__ x, gbn_layout XL) {
    extern __shared__ float2 st_cs[];
    constexpr int KP = kSenseSeg / kThreads;
    const Geom &g = a.g;
    const int D = g.dim;
    const int ml = last_axis(a.m, D), Ld = last_axis(g.nf, D);
    const float *tl = last_axis(a.tab, D);
    const BandRow r = band_row(a, dc, blockIdx.x, false);
    const int SP = dc.seg + 1;
    const bool sens_coil_fast = SL.coil_stride < SL.elem_stride;

    float2 acc[KP];
    int cell[KP];
#pragma unroll
    for (int k = 0; k < KP; ++k) {
        acc[k] = make_float2(0.f, 0.f);
        const int kk = threadIdx.x + k * kThreads;
        cell[k] = kk < r.seg_len ? grid_index(r.i0 + kk, ml, Ld) : 0;
    }
    const float2 *rows = grid + r.grp * g.n_coil * g.G + r.gbase * Ld;

    for (int c0 = 0; c0 < g.n_coil; c0 += dc.cc) {
        const int n_cc = min(dc.cc, g.n_coil - c0);
        __syncthreads();  // previous chunk consumed
        const int n = n_cc * r.seg_len;
        for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
            int cc, k;
            if (sens_coil_fast) {
                k = idx / n_cc;
                cc = idx - k * n_cc;
            } else {
                cc = idx / r.seg_len;
                k = idx - cc * r.seg_len;
            }
            st_cs[cc * SP + k] =
                sens[(r.p * ml + r.i0 + k) * SL.elem_stride + (int64_t)(c0 + cc) * SL.coil_stride];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < KP; ++k) {
            const int kk = threadIdx.x + k * kThreads;
            if (kk < r.seg_len) {  // a guard, not a break: the loop stays unrolled, acc in registers
                float ax = acc[k].x, ay = acc[k].y;
                for (int cc = 0; cc < n_cc; ++cc) {
                    const float2 v = rows[(int64_t)(c0 + cc) * g.G + cell[k]];
                    const float2 sv = st_cs[cc * SP + kk];
                    ax += sv.x * v.x + sv.y * v.y;
                    ay += sv.x * v.y - sv.y * v.x;
                }
                acc[k] = make_float2(ax, ay);
            }
        }
    }

    const float s = a.grp_scale ? r.s * a.grp_scale[r.grp] : r.s;
    float2 *dst = x + r.grp * XL.traj_stride;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
        const int kk = threadIdx.x + k * kThreads;
        if (kk < r.seg_len) {
            const int i = r.i0 + kk;
            const float f = s * tl[i];
            dst[(r.p * ml + i) * XL.elem_stride] = make_float2(acc[k].x * f, acc[k].y * f);
        }
    }
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// seg_cap: longest segment of the last image dim per block; chunked: coil chunks are
// separate blocks (pad, crop) rather than a loop inside the block (crop_sense);
// zero: the launch also fills the out-of-band slabs (pad)
Decomp make_decomp(const DeapodArgs &a, int seg_cap, bool chunked, bool zero, bool coil_fast, int min_cc = 1) {
    const Geom &g = a.g;
    const int D = g.dim;
    Decomp dc{};
    dc.n_outer = 1;
    for (int d = 0; d < D - 1; ++d) dc.n_outer *= a.m[d];
    const int ml = a.m[D - 1];
    dc.seg = ml < seg_cap ? ml : seg_cap;
    dc.nseg = (int)ceil_div(ml, dc.seg);
    dc.cc = (int)std::max<int64_t>(1, std::min<int64_t>(g.n_coil, kStageElems / (dc.seg + 1)));
    if (chunked) {
        // equal chunks (16 coils: 8 + 8, not 15 + 1), and more of them while the launch has
        // few rows (a 2-D image of a few hundred rows): enough blocks to fill the GPU, down
        // to min_cc coils per chunk
        int64_t ncc = ceil_div(g.n_coil, dc.cc);
        const int64_t rows = (int64_t)g.n_traj * dc.n_outer * dc.nseg;
        while (rows * ncc < kMinBandBlocks && ncc < g.n_coil && ceil_div(g.n_coil, 2 * ncc) >= min_cc) ncc *= 2;
        dc.cc = (int)ceil_div(g.n_coil, std::min<int64_t>(ncc, g.n_coil));
    }
    dc.ncc = chunked ? (int)ceil_div(g.n_coil, dc.cc) : 1;
    dc.nband = (int64_t)g.n_traj * dc.n_outer * dc.ncc * dc.nseg;
    dc.coil_fast = coil_fast;
    if (zero && D >= 2) {
        const int64_t n_inst = (int64_t)g.n_coil * g.n_traj;
        dc.x_len = (int64_t)(g.nf[0] - a.m[0]) * (g.G / g.nf[0]);
        dc.x_chunks = ceil_div(dc.x_len, kZeroChunk);
        dc.nzero = n_inst * dc.x_chunks;
        if (D == 3) {
            dc.y_len = (int64_t)(g.nf[1] - a.m[1]) * g.nf[2];
            dc.y_chunks = ceil_div(dc.y_len, kZeroChunk);
            dc.nzero += n_inst * a.m[0] * dc.y_chunks;
        }
    }
    return dc;
}

size_t stage_bytes(const Decomp &dc) { return (size_t)dc.cc * (dc.seg + 1) * sizeof(float2); }

bool empty(const DeapodArgs &a) {
    if ((int64_t)a.g.n_coil * a.g.n_traj == 0) return true;
    for (int d = 0; d < a.g.dim; ++d)
        if (a.m[d] == 0) return true;
    return false;
}

// Coils per chunk for an image in host memory (pinned, read or written by the kernel over
// the host link): with coils fastest, 8 coils keep each pixel's 64-byte run in one block;
// 2-coil chunks (16-byte pieces) made the c2 host-buffer step 25 % slower.
// The query is skipped while the stream is being captured into a graph (host-buffer calls
// are never captured).
int host_min_cc(const void *img, bool coil_fast, int n_coil, cudaStream_t s) {
    if (!coil_fast) return 1;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return 1;
    }
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, img) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return at.type == cudaMemoryTypeHost ? std::min(8, n_coil) : 1;
}

cudaError_t check_blocks(int64_t n) {
    return n > 0x7FFFFFFF ? cudaErrorInvalidConfiguration : cudaSuccess;
}

}  // namespace

cudaError_t launch_build_tables(int dim, const int m[3], const int nf[3], double tau, float *tab0, float *tab1,
                                float *tab2, cudaStream_t s) {
    float *tabs[3] = {tab0, tab1, tab2};
    for (int d = 0; d < 3; ++d) {
        if (d < dim)
            k_build_table<<<(m[d] + 255) / 256, 256, 0, s>>>(m[d], nf[d], tau, tabs[d]);
        else
            k_fill_one<<<1, 1, 0, s>>>(tabs[d]);
    }
    return cudaGetLastError();
}

cudaError_t launch_pad(const DeapodArgs &a, const float2 *img, gbn_layout L, float2 *grid, cudaStream_t s) {
    NvtxRange range("gbn pad");
    if (empty(a)) return cudaSuccess;
    const bool cf = L.coil_stride < L.elem_stride;
    const Decomp dc = make_decomp(a, kStageElems - 1, true, true, cf, host_min_cc(img, cf, a.g.n_coil, s));
    const int64_t nb = dc.nband + dc.nzero;
    if (cudaError_t e = check_blocks(nb)) return e;
    k_pad<ImageSrc><<<(unsigned)nb, kThreads, stage_bytes(dc), s>>>(a, dc, ImageSrc{img, L}, grid);
    return cudaGetLastError();
}

cudaError_t launch_crop(const DeapodArgs &a, const float2 *grid, float2 *img, gbn_layout L, cudaStream_t s) {
    NvtxRange range("gbn crop");
    if (empty(a)) return cudaSuccess;
    const bool cf = L.coil_stride < L.elem_stride;
    const Decomp dc = make_decomp(a, kStageElems - 1, true, false, cf, host_min_cc(img, cf, a.g.n_coil, s));
    if (cudaError_t e = check_blocks(dc.nband)) return e;
    k_crop<<<(unsigned)dc.nband, kThreads, stage_bytes(dc), s>>>(a, dc, grid, img, L);
    return cudaGetLastError();
}

cudaError_t launch_pad_sense(const DeapodArgs &a, const float2 *x, gbn_layout XL, const float2 *sens,
                             gbn_layout SL, float2 *grid, cudaStream_t s) {
    NvtxRange range("gbn pad (SENSE)");
    if (empty(a)) return cudaSuccess;
    const bool cf = SL.coil_stride < SL.elem_stride;
    const Decomp dc = make_decomp(a, kStageElems - 1, true, true, cf, host_min_cc(x, cf, a.g.n_coil, s));
    const int64_t nb = dc.nband + dc.nzero;
    if (cudaError_t e = check_blocks(nb)) return e;
    k_pad<SenseSrc><<<(unsigned)nb, kThreads, stage_bytes(dc), s>>>(a, dc, SenseSrc{x, XL, sens, SL}, grid);
    return cudaGetLastError();
}

cudaError_t launch_crop_sense(const DeapodArgs &a, const float2 *grid, const float2 *sens, gbn_layout SL,
                              float2 *x, gbn_layout XL, cudaStream_t s) {
    NvtxRange range("gbn crop (SENSE)");
    if (empty(a)) return cudaSuccess;
    const Decomp dc = make_decomp(a, kSenseSeg, false, false, false);
    if (cudaError_t e = check_blocks(dc.nband)) return e;
    k_crop_sense<<<(unsigned)dc.nband, kThreads, stage_bytes(dc), s>>>(a, dc, grid, sens, SL, x, XL);
    return cudaGetLastError();
}

}  // namespace gbn
