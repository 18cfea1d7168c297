// ESPIRiT's pixel-wise eigen step (espirit/espirit_func.py:72-81 (2-D), :186-196 (3-D)):
// for every pixel the ESPIRiT kernels in image space form A (nsv x nc, one row per kept
// singular vector); the reference takes the SVD of vvH = A^T conj(A) (nc x nc, Hermitian,
// positive semi-definite) and keeps its largest singular value (the eigenvalue map) and
// the conjugate of the first row of V^H, i.e. the top eigenvector.
//
// One warp per pixel: lane c accumulates row c of vvH in registers (sum over the kernels of
// A[k][c] conj(A[k][d]), A[k][d] broadcast by shuffles), then runs power iterations on it,
// starting from the column of the largest diagonal entry.  The eigenvalue is the Rayleigh
// quotient v^H vvH v.  The reference's eigenvector phase is LAPACK's (arbitrary per pixel);
// here it is fixed: coil 0's component real and non-negative (the first non-zero coil's when
// coil 0 vanishes), which makes the maps continuous where the reference's are not.
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
__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(32 * kEspWarps) k_espirit_eigen(const float2 *__restrict__ a, int64_t n_pix,
                                                                  int nsv, int nc, int n_iter,
                                                                  float2 *__restrict__ vmap,
                                                                  float *__restrict__ smap) {
    const int lane = threadIdx.x & 31;
    const int64_t pix = (int64_t)blockIdx.x * kEspWarps + (threadIdx.x >> 5);
    if (pix >= n_pix) return;  // warp-uniform
    const bool act = lane < nc;
    // row `lane` of vvH
    float2 m[kEspMaxCoils];
#pragma unroll
    for (int d = 0; d < kEspMaxCoils; ++d) m[d] = make_float2(0.f, 0.f);
    const float2 *ap = a + pix * (int64_t)nsv * nc;
    for (int k = 0; k < nsv; ++k) {
        const float2 mine = act ? ap[(int64_t)k * nc + lane] : make_float2(0.f, 0.f);
#pragma unroll
        for (int d = 0; d < kEspMaxCoils; ++d) {
            if (d >= nc) break;
            float2 o;
            o.x = __shfl_sync(0xffffffffu, mine.x, d);
            o.y = __shfl_sync(0xffffffffu, mine.y, d);
            const float2 t = cmul_conj(mine, o);
            m[d].x += t.x;
            m[d].y += t.y;
        }
    }
    // start: the column of the largest diagonal entry (the row's conjugate, by symmetry)
    float diag = 0.f;
#pragma unroll
    for (int d = 0; d < kEspMaxCoils; ++d)
        if (d == lane) diag = m[d].x;
    float best = act ? diag : -1.f;
    int arg = lane;
    for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
        if (ob > best || (ob == best && oa < arg)) {
            best = ob;
            arg = oa;
        }
    }
    // column `arg` of vvH: entry `lane` is vvH[lane][arg] = m[arg] of this lane's row
    float2 v = make_float2(0.f, 0.f);
#pragma unroll
    for (int d = 0; d < kEspMaxCoils; ++d)
        if (d == arg) v = act ? m[d] : make_float2(0.f, 0.f);
    float nrm = sqrtf(warp_sum(v.x * v.x + v.y * v.y));
    if (nrm > 0.f) {
        v.x /= nrm;
        v.y /= nrm;
    }
    float lam = 0.f;
    for (int it = 0; it <= n_iter; ++it) {
        float2 w = make_float2(0.f, 0.f);
#pragma unroll
        for (int d = 0; d < kEspMaxCoils; ++d) {
            if (d >= nc) break;
            float2 vd;
            vd.x = __shfl_sync(0xffffffffu, v.x, d);
            vd.y = __shfl_sync(0xffffffffu, v.y, d);
            const float2 t = cmul(m[d], vd);
            w.x += t.x;
            w.y += t.y;
        }
        if (!act) w = make_float2(0.f, 0.f);
        // Rayleigh quotient v^H (vvH v) with the current (unit) v
        lam = warp_sum(v.x * w.x + v.y * w.y);
        if (it == n_iter) break;
        nrm = sqrtf(warp_sum(w.x * w.x + w.y * w.y));
        if (!(nrm > 0.f)) break;
        v = make_float2(w.x / nrm, w.y / nrm);
    }
    // canonical phase: the first coil with a non-zero component made real and positive
    const float mag2 = v.x * v.x + v.y * v.y;
    const unsigned nz = __ballot_sync(0xffffffffu, act && mag2 > 0.f);
    if (nz) {
        const int src = __ffs(nz) - 1;
        const float px = __shfl_sync(0xffffffffu, v.x, src), py = __shfl_sync(0xffffffffu, v.y, src);
        const float pm = sqrtf(px * px + py * py);
        const float2 ph = make_float2(px / pm, -py / pm);  // conj(v_src) / |v_src|
        v = cmul(v, ph);
    }
    if (act) vmap[pix * nc + lane] = v;
    if (lane == 0) smap[pix] = lam;
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
    const int64_t blocks = (n_pix + kEspWarps - 1) / kEspWarps;
    if (blocks > 0x7fffffff) return record_error(GBN_ERR_CAPACITY, "ESPIRiT eigen: too many pixels");
    k_espirit_eigen<<<(unsigned)blocks, 32 * kEspWarps, 0, (cudaStream_t)stream>>>(
        (const float2 *)a, n_pix, nsv, nc, n_iter, (float2 *)vmap, smap);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return record_error(GBN_ERR_CUDA, (std::string("ESPIRiT eigen: ") + cudaGetErrorString(e)).c_str());
    return GBN_OK;
}
