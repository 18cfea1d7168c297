// ESPIRiT's pixel-wise eigen step (espirit/espirit_func.py:72-81 (2-D), :186-196 (3-D)):
// for every pixel the ESPIRiT kernels in image space form A (nsv x nc, one row per kept
// singular vector); the reference takes the SVD of vvH = A^T conj(A) (nc x nc, Hermitian,
// positive semi-definite) and keeps its largest singular value (the eigenvalue map) and
// the conjugate of the first row of V^H, i.e. the top eigenvector.
//
// Pixels in lane groups: a group of GS lanes (GS = the power of two >= nc, at least 4) takes
// one pixel, so a warp works on 32 / GS pixels at once.  Lane c of a group accumulates row c
// of vvH in registers (sum over the kernels of A[k][c] conj(A[k][d]), A[k][d] broadcast by
// shuffles within the group), then runs power iterations on it, starting from the column of
// the largest diagonal entry.  The eigenvalue is the Rayleigh quotient v^H vvH v.  The
// reference's eigenvector phase is LAPACK's (arbitrary per pixel); here it is fixed: coil 0's
// component real and non-negative (the first non-zero coil's when coil 0 vanishes), which
// makes the maps continuous where the reference's are not.  Every shuffle runs with the whole
// warp converged: pixels past the end and converged iterations compute on zeros instead of
// leaving the loop.
#include <cmath>
#include <string>

#include "common.cuh"

namespace gbn {
namespace {

constexpr int kEspMaxCoils = 32;
constexpr int kEspWarps = 8;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmul_conj(float2 a, float2 b) {  // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <int GS>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = GS / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int GS>
__global__ void __launch_bounds__(32 * kEspWarps) k_espirit_eigen(const float2 *__restrict__ a, int64_t n_pix,
                                                                  int nsv, int nc, int n_iter,
                                                                  float2 *__restrict__ vmap,
                                                                  float *__restrict__ smap) {
    constexpr int PPW = 32 / GS;                    // pixels per warp
    const int lane = threadIdx.x & 31;
    const int c = lane % GS;                        // coil (row of vvH) within the group
    const int grp0 = lane - c;                      // first lane of the group
    const int64_t pix = ((int64_t)blockIdx.x * kEspWarps + (threadIdx.x >> 5)) * PPW + lane / GS;
    const bool valid = pix < n_pix;
    const bool act = valid && c < nc;
    // row c of vvH
    float2 m[GS];
#pragma unroll
    for (int d = 0; d < GS; ++d) m[d] = make_float2(0.f, 0.f);
    const float2 *ap = a + (valid ? pix : 0) * (int64_t)nsv * nc;
    for (int k = 0; k < nsv; ++k) {
        const float2 mine = act ? ap[(int64_t)k * nc + c] : make_float2(0.f, 0.f);
#pragma unroll
        for (int d = 0; d < GS; ++d) {
            float2 o;
            o.x = __shfl_sync(0xffffffffu, mine.x, grp0 + d);
            o.y = __shfl_sync(0xffffffffu, mine.y, grp0 + d);
            const float2 t = cmul_conj(mine, o);
            m[d].x += t.x;
            m[d].y += t.y;
        }
    }
    // start: the column of the largest diagonal entry (the row's conjugate, by symmetry)
    float diag = 0.f;
#pragma unroll
    for (int d = 0; d < GS; ++d)
        if (d == c) diag = m[d].x;
    float best = act ? diag : -1.f;
    int arg = c;
#pragma unroll
    for (int o = GS / 2; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
        if (ob > best || (ob == best && oa < arg)) {
            best = ob;
            arg = oa;
        }
    }
    // column `arg` of vvH: entry c is vvH[c][arg] = m[arg] of this lane's row
    float2 v = make_float2(0.f, 0.f);
#pragma unroll
    for (int d = 0; d < GS; ++d)
        if (d == arg) v = act ? m[d] : make_float2(0.f, 0.f);
    float nrm = sqrtf(group_sum<GS>(v.x * v.x + v.y * v.y));
    if (nrm > 0.f) {
        v.x /= nrm;
        v.y /= nrm;
    }
    float lam = 0.f;
    for (int it = 0; it <= n_iter; ++it) {
        float2 w = make_float2(0.f, 0.f);
#pragma unroll
        for (int d = 0; d < GS; ++d) {
            float2 vd;
            vd.x = __shfl_sync(0xffffffffu, v.x, grp0 + d);
            vd.y = __shfl_sync(0xffffffffu, v.y, grp0 + d);
            const float2 t = cmul(m[d], vd);
            w.x += t.x;
            w.y += t.y;
        }
        if (!act) w = make_float2(0.f, 0.f);
        // Rayleigh quotient v^H (vvH v) with the current (unit) v
        lam = group_sum<GS>(v.x * w.x + v.y * w.y);
        if (it == n_iter) break;                    // uniform across the warp
        nrm = sqrtf(group_sum<GS>(w.x * w.x + w.y * w.y));
        // a vanishing product leaves v (and so w = 0 and lam = 0) unchanged from here on
        if (nrm > 0.f) v = make_float2(w.x / nrm, w.y / nrm);
    }
    // canonical phase: the first coil with a non-zero component made real and positive
    const float mag2 = v.x * v.x + v.y * v.y;
    const unsigned nz = (__ballot_sync(0xffffffffu, act && mag2 > 0.f) >> grp0) & (GS == 32 ? 0xffffffffu : ((1u << GS) - 1u));
    const int src = nz ? __ffs(nz) - 1 : 0;
    const float px = __shfl_sync(0xffffffffu, v.x, grp0 + src), py = __shfl_sync(0xffffffffu, v.y, grp0 + src);
    if (nz) {
        const float pm = sqrtf(px * px + py * py);
        const float2 ph = make_float2(px / pm, -py / pm);  // conj(v_src) / |v_src|
        v = cmul(v, ph);
    }
    if (act) vmap[pix * nc + c] = v;
    if (valid && c == 0) smap[pix] = lam;
}

}  // namespace
}  // namespace gbn

using namespace gbn;

int gbn_espirit_eigen(const void *a, int64_t n_pix, int32_t nsv, int32_t nc, int32_t n_iter, void *vmap, float *smap,
                      gbn_stream_t stream) {
    if (n_pix < 0 || nsv < 0 || nc < 1 || n_iter < 0) return record_error(GBN_ERR_ARG, "ESPIRiT eigen: bad size");
    if (nc > kEspMaxCoils) return record_error(GBN_ERR_CAPACITY, "ESPIRiT eigen: more than 32 coils");
    if (n_pix == 0) return GBN_OK;
    if ((!a && nsv > 0) || !vmap || !smap) return record_error(GBN_ERR_ARG, "ESPIRiT eigen: null buffer");
    const int gs = nc <= 4 ? 4 : nc <= 8 ? 8 : nc <= 16 ? 16 : 32;
    const int64_t per_block = (int64_t)kEspWarps * (32 / gs);
    const int64_t blocks = (n_pix + per_block - 1) / per_block;
    if (blocks > 0x7fffffff) return record_error(GBN_ERR_CAPACITY, "ESPIRiT eigen: too many pixels");
    const dim3 grid((unsigned)blocks), block(32 * kEspWarps);
    cudaStream_t s = (cudaStream_t)stream;
    const float2 *ap = (const float2 *)a;
    if (gs == 4) k_espirit_eigen<4><<<grid, block, 0, s>>>(ap, n_pix, nsv, nc, n_iter, (float2 *)vmap, smap);
    else if (gs == 8) k_espirit_eigen<8><<<grid, block, 0, s>>>(ap, n_pix, nsv, nc, n_iter, (float2 *)vmap, smap);
    else if (gs == 16) k_espirit_eigen<16><<<grid, block, 0, s>>>(ap, n_pix, nsv, nc, n_iter, (float2 *)vmap, smap);
    else k_espirit_eigen<32><<<grid, block, 0, s>>>(ap, n_pix, nsv, nc, n_iter, (float2 *)vmap, smap);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return record_error(GBN_ERR_CUDA, (std::string("ESPIRiT eigen: ") + cudaGetErrorString(e)).c_str());
    return GBN_OK;
}
