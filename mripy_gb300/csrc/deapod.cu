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
#include "common.cuh"

namespace gbn {

namespace {

__global__ void k_build_table(int m, int nf, double tau, float *tab) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const double pi = 3.14159265358979323846;
    double k = (double)(i - m / 2);
    tab[i] = (float)(sqrt(pi / tau) * exp(tau * k * k) / (double)nf);
}

__global__ void k_fill_one(float *tab) { tab[0] = 1.f; }

// image index for grid index gi along one dim (-1: outside the image band)
__device__ __forceinline__ int img_index(int gi, int m, int nf) {
    const int h = m / 2;
    if (gi < m - h) return gi + h;
    if (gi >= nf - h) return gi - nf + h;
    return -1;
}

__global__ void k_pad(DeapodArgs a, const float2 *__restrict__ img, gbn_layout L, float2 *__restrict__ grid,
                      int64_t total) {
    const Geom &g = a.g;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t inst = t / g.G;
        const int64_t cell = t - inst * g.G;
        const int g2 = (int)(cell % g.nf[2]);
        const int g1 = (int)((cell / g.nf[2]) % g.nf[1]);
        const int g0 = (int)(cell / ((int64_t)g.nf[2] * g.nf[1]));
        const int i0 = img_index(g0, a.m[0], g.nf[0]);
        const int i1 = img_index(g1, a.m[1], g.nf[1]);
        const int i2 = img_index(g2, a.m[2], g.nf[2]);
        float2 out = make_float2(0.f, 0.f);
        if ((i0 | i1 | i2) >= 0) {
            const int grp = (int)(inst / g.n_coil), coil = (int)(inst - (int64_t)grp * g.n_coil);
            const int64_t p = ((int64_t)i0 * a.m[1] + i1) * a.m[2] + i2;
            const float2 v = img[grp * L.traj_stride + coil * L.coil_stride + p * L.elem_stride];
            const float s = a.tab[0][i0] * a.tab[1][i1] * a.tab[2][i2];
            out = make_float2(v.x * s, v.y * s);
        }
        grid[t] = out;
    }
}

__global__ void k_crop(DeapodArgs a, const float2 *__restrict__ grid, float2 *__restrict__ img, gbn_layout L,
                       int64_t total) {
    const Geom &g = a.g;
    const int64_t P = (int64_t)a.m[0] * a.m[1] * a.m[2];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t inst = t / P;
        const int64_t p = t - inst * P;
        const int i2 = (int)(p % a.m[2]);
        const int i1 = (int)((p / a.m[2]) % a.m[1]);
        const int i0 = (int)(p / ((int64_t)a.m[2] * a.m[1]));
        int g0 = i0 - a.m[0] / 2; g0 += g0 < 0 ? g.nf[0] : 0;
        int g1 = i1 - a.m[1] / 2; g1 += g1 < 0 ? g.nf[1] : 0;
        int g2 = i2 - a.m[2] / 2; g2 += g2 < 0 ? g.nf[2] : 0;
        const int grp = (int)(inst / g.n_coil), coil = (int)(inst - (int64_t)grp * g.n_coil);
        const float2 v = grid[inst * g.G + ((int64_t)g0 * g.nf[1] + g1) * g.nf[2] + g2];
        float s = a.tab[0][i0] * a.tab[1][i1] * a.tab[2][i2];
        if (a.grp_scale) s *= a.grp_scale[grp];
        img[grp * L.traj_stride + coil * L.coil_stride + p * L.elem_stride] = make_float2(v.x * s, v.y * s);
    }
}

// grid[(grp, coil)] = pad(deapod * x[grp] * sens[coil])
__global__ void k_pad_sense(DeapodArgs a, const float2 *__restrict__ x, gbn_layout XL,
                            const float2 *__restrict__ sens, gbn_layout SL, float2 *__restrict__ grid,
                            int64_t total) {
    const Geom &g = a.g;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t inst = t / g.G;
        const int64_t cell = t - inst * g.G;
        const int g2 = (int)(cell % g.nf[2]);
        const int g1 = (int)((cell / g.nf[2]) % g.nf[1]);
        const int g0 = (int)(cell / ((int64_t)g.nf[2] * g.nf[1]));
        const int i0 = img_index(g0, a.m[0], g.nf[0]);
        const int i1 = img_index(g1, a.m[1], g.nf[1]);
        const int i2 = img_index(g2, a.m[2], g.nf[2]);
        float2 out = make_float2(0.f, 0.f);
        if ((i0 | i1 | i2) >= 0) {
            const int grp = (int)(inst / g.n_coil), coil = (int)(inst - (int64_t)grp * g.n_coil);
            const int64_t p = ((int64_t)i0 * a.m[1] + i1) * a.m[2] + i2;
            const float2 v = x[grp * XL.traj_stride + p * XL.elem_stride];
            const float2 sv = sens[coil * SL.coil_stride + p * SL.elem_stride];
            const float s = a.tab[0][i0] * a.tab[1][i1] * a.tab[2][i2];
            out = make_float2((v.x * sv.x - v.y * sv.y) * s, (v.x * sv.y + v.y * sv.x) * s);
        }
        grid[t] = out;
    }
}

// x[grp] = sum_coil conj(sens[coil]) * crop(deapod * grid[(grp, coil)])
__global__ void k_crop_sense(DeapodArgs a, const float2 *__restrict__ grid, const float2 *__restrict__ sens,
                             gbn_layout SL, float2 *__restrict__ x, gbn_layout XL, int64_t total) {
    const Geom &g = a.g;
    const int64_t P = (int64_t)a.m[0] * a.m[1] * a.m[2];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t grp = t / P;
        const int64_t p = t - grp * P;
        const int i2 = (int)(p % a.m[2]);
        const int i1 = (int)((p / a.m[2]) % a.m[1]);
        const int i0 = (int)(p / ((int64_t)a.m[2] * a.m[1]));
        int g0 = i0 - a.m[0] / 2; g0 += g0 < 0 ? g.nf[0] : 0;
        int g1 = i1 - a.m[1] / 2; g1 += g1 < 0 ? g.nf[1] : 0;
        int g2 = i2 - a.m[2] / 2; g2 += g2 < 0 ? g.nf[2] : 0;
        const int64_t cell = ((int64_t)g0 * g.nf[1] + g1) * g.nf[2] + g2;
        float ax = 0.f, ay = 0.f;
        for (int coil = 0; coil < g.n_coil; ++coil) {
            const float2 v = grid[(grp * g.n_coil + coil) * g.G + cell];
            const float2 sv = sens[coil * SL.coil_stride + p * SL.elem_stride];
            ax += sv.x * v.x + sv.y * v.y;
            ay += sv.x * v.y - sv.y * v.x;
        }
        float s = a.tab[0][i0] * a.tab[1][i1] * a.tab[2][i2];
        if (a.grp_scale) s *= a.grp_scale[grp];
        x[grp * XL.traj_stride + p * XL.elem_stride] = make_float2(ax * s, ay * s);
    }
}

inline unsigned grid_blocks(int64_t n, int th) {
    int64_t b = (n + th - 1) / th;
    const int64_t cap = 152 * 32;  // grid-stride beyond a few waves of the 152 SMs
    return (unsigned)(b < cap ? (b > 0 ? b : 1) : cap);
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
    const int64_t total = a.g.G * (int64_t)a.g.n_coil * a.g.n_traj;
    k_pad<<<grid_blocks(total, 256), 256, 0, s>>>(a, img, L, grid, total);
    return cudaGetLastError();
}

cudaError_t launch_crop(const DeapodArgs &a, const float2 *grid, float2 *img, gbn_layout L, cudaStream_t s) {
    const int64_t total = (int64_t)a.m[0] * a.m[1] * a.m[2] * a.g.n_coil * a.g.n_traj;
    k_crop<<<grid_blocks(total, 256), 256, 0, s>>>(a, grid, img, L, total);
    return cudaGetLastError();
}

cudaError_t launch_pad_sense(const DeapodArgs &a, const float2 *x, gbn_layout XL, const float2 *sens,
                             gbn_layout SL, float2 *grid, cudaStream_t s) {
    const int64_t total = a.g.G * (int64_t)a.g.n_coil * a.g.n_traj;
    k_pad_sense<<<grid_blocks(total, 256), 256, 0, s>>>(a, x, XL, sens, SL, grid, total);
    return cudaGetLastError();
}

cudaError_t launch_crop_sense(const DeapodArgs &a, const float2 *grid, const float2 *sens, gbn_layout SL,
                              float2 *x, gbn_layout XL, cudaStream_t s) {
    const int64_t total = (int64_t)a.m[0] * a.m[1] * a.m[2] * a.g.n_traj;
    k_crop_sense<<<grid_blocks(total, 256), 256, 0, s>>>(a, grid, sens, SL, x, XL, total);
    return cudaGetLastError();
}

}  // namespace gbn
