// Interp (type-2 gridding) and trajectory-gradient launchers.
//
// 2-D with at most 16 taps per dimension: k_interp2d (one warp per sample, coils across
// lanes).  Otherwise (1-D, 3-D, wide stencils): k_interp (one thread per sample).
#include "dispatch.cuh"
#include "grid2d_kernels.cuh"
#include "grid3d_kernels.cuh"

namespace gbn {

static bool use_2d_path(const Geom &g) { return g.dim == 2 && g.W <= 16; }

size_t interp_smem_bytes(const Geom &g, int coil_group) {
    if (use_2d_path(g)) return interp2d_smem_bytes(g, coil_group);
    size_t cells = 1;
    for (int d = 0; d < g.dim; ++d) cells *= (size_t)(g.tile[d] + g.W - 1);
    return cells * (size_t)coil_group * sizeof(float2);
}

static size_t grad_smem_bytes(const Geom &g, int coil_group) {
    size_t cells = 1;
    for (int d = 0; d < g.dim; ++d) cells *= (size_t)(g.tile[d] + g.W - 1);
    return cells * (size_t)coil_group * sizeof(float2);
}

cudaError_t launch_interp(const InterpArgs &a, int64_t n_sub, int coil_group, int threads, cudaStream_t s) {
    if (n_sub == 0) return cudaSuccess;
    const size_t smem = interp_smem_bytes(a.g, coil_group);
    const dim3 grid((unsigned)n_sub, (unsigned)((a.g.n_coil + coil_group - 1) / coil_group));
    cudaError_t err = cudaSuccess;
    if (use_2d_path(a.g)) {
        GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
            auto kern = k_interp2d<WT, CG>;
            err = set_smem(kern, smem);
            if (err == cudaSuccess) {
                kern<<<grid, threads, smem, s>>>(a);
                err = cudaGetLastError();
            }
        }));
        return err;
    }
    if (a.g.dim == 3 && a.g.W <= 16) {
        GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
            auto kern = k_interp3d<WT, CG>;
            err = set_smem(kern, smem);
            if (err == cudaSuccess) {
                kern<<<grid, threads > 256 ? 256 : threads, smem, s>>>(a);
                err = cudaGetLastError();
            }
        }));
        return err;
    }
    GBN_DISPATCH_D(a.g.dim, GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
        auto kern = k_interp<D, WT, CG>;
        err = set_smem(kern, smem);
        if (err == cudaSuccess) {
            kern<<<grid, threads, smem, s>>>(a);
            err = cudaGetLastError();
        }
    })));
    return err;
}

cudaError_t launch_interp_grad(const GradArgs &a, int64_t n_sub, int coil_group, int threads, cudaStream_t s) {
    if (n_sub == 0) return cudaSuccess;
    const size_t smem = grad_smem_bytes(a.g, coil_group);
    const dim3 grid((unsigned)n_sub, (unsigned)((a.g.n_coil + coil_group - 1) / coil_group));
    // dw/dx = w * (-2 beta d / h) with beta = beta2 / log2(e), h = 2 pi / nf
    float dsc[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < a.g.dim; ++d) {
        const double beta = (double)a.g.beta2[d] / 1.4426950408889634;
        const double h = 6.283185307179586 / a.g.nf[d];
        dsc[d] = (float)(-2.0 * beta / h);
    }
    cudaError_t err = cudaSuccess;
    GBN_DISPATCH_D(a.g.dim, GBN_DISPATCH_W(a.g.W, GBN_DISPATCH_CG(coil_group, {
        auto kern = k_interp_grad<D, WT, CG>;
        err = set_smem(kern, smem);
        if (err == cudaSuccess) {
            kern<<<grid, threads > 256 ? 256 : threads, smem, s>>>(a, dsc[0], dsc[1], dsc[2]);
            err = cudaGetLastError();
        }
    })));
    return err;
}

}  // namespace gbn
