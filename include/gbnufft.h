/*
 * gbnufft: Gaussian-gridding NUFFT for NVIDIA GB300 (sm_103a), C ABI.
 *
 * Drop-in engine behind mripy's NUFFT function API (peng-cao/mripy
 * fft/nufft_func.py, fft/nufft_func_cuda.py) and NUFFT operator classes
 * (pics/operators_class.py, pics/operators_cuda_class.py).  Every entry point
 * takes plain pointers, sizes and a cudaStream_t, returns an int status
 * (GBN_OK == 0) and throws nothing.  Device pointers are marked "device";
 * the gbn_nufft*_gaussker and *_host entry points take host pointers.
 *
 * Conventions shared with the reference (nufft_func.py):
 *  - coordinates x_j are radians; they are scaled by df and wrapped mod 2*pi;
 *  - nspread, oversampled grid nf and tau follow _compute_{1,2,3}d_grid_params
 *    (nufft_func.py:198-249; the 3-D operator clamps nspread to [3, 6]);
 *  - type-1 (adjoint)  F_k = (1/M) sum_j c_j exp(+s i k.x_j),  s = sign(iflag);
 *  - type-2 (forward)  c_j = sum_k F_k exp(-s i k.x_j);
 *  - type-21 (normal)  (1/M) A^H D A F, D = dcf (3-D) or identity;
 *  - image index i <-> frequency k = i - m/2 (m//2 in Python), row-major
 *    (x slowest, then y, then z), as numpy arrays of shape (ms, mt[, mu]).
 * Arithmetic: complex64 data, FP32 stencil arithmetic and accumulation; FP64
 * only for coordinate reduction, parameter and deapodisation-table set-up.
 */
#ifndef GBNUFFT_H
#define GBNUFFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef GBN_STREAM_T_DEFINED
#define GBN_STREAM_T_DEFINED
typedef struct CUstream_st *gbn_stream_t; /* == cudaStream_t; NULL = legacy default stream */
#endif

/* status codes */
#define GBN_OK 0
#define GBN_ERR_ARG 1       /* invalid argument (shape, size, pointer, parameter) */
#define GBN_ERR_ALLOC 2     /* device or pinned-host allocation failed */
#define GBN_ERR_CUDA 3      /* CUDA runtime error (message via gbn_last_error) */
#define GBN_ERR_CUFFT 4     /* cuFFT error */
#define GBN_ERR_STATE 5     /* call order: e.g. transform before gbn_set_points */
#define GBN_ERR_CAPACITY 6  /* size beyond a documented limit */
#define GBN_ERR_INTERNAL 7  /* unexpected host-side failure */
#define GBN_ERR_TIMEOUT 8   /* a kernel's bounded wait gave up (reported by gbn_plan_status) */

#define GBN_COORD_F32 0
#define GBN_COORD_F64 1

#define GBN_FFT_FORWARD (-1) /* exp(-i ...), numpy.fft.fftn, unnormalised */
#define GBN_FFT_INVERSE (+1) /* exp(+i ...), unnormalised                  */

#define GBN_BAND_INPUT 1  /* gbn_fft_band: the grid is zero outside the image band (as the pad leaves it) */
#define GBN_BAND_OUTPUT 2 /* gbn_fft_band: only the image band of the result is read (as the crop reads it) */

typedef struct gbn_plan gbn_plan;   /* opaque */
typedef struct gbn_graph gbn_graph; /* opaque captured CUDA graph */

typedef struct {
    int32_t dim;            /* 1, 2 or 3 */
    int32_t ms, mt, mu;     /* image size along x, y, z (unused dims: 1) */
    double eps;             /* requested accuracy; selects nspread, ratio, tau */
    int32_t max_nspread;    /* 0 = no clamp (1-D/2-D); 6 = the 3-D reference clamp */
    int32_t iflag;          /* sign convention (see above) */
    double df;              /* coordinate scale */
    int32_t n_coil;         /* instances that share one trajectory (coils) */
    int32_t n_traj;         /* trajectory groups (frames/slices), ragged sample counts */
    /* tuning (0 = library default; the autotuner fills these) */
    int32_t spread_tile[3]; /* output tile of the spread kernel, cells per dim */
    int32_t interp_tile[3]; /* home bin of the interp kernel, cells per dim */
    int32_t max_subproblem; /* samples per thread block before a bin is split */
    int32_t coil_group;     /* coils per spread thread block: 1, 2, 4 or 8 */
    int32_t threads;        /* threads per spread block: 128, 256 or 512 */
    int32_t interp_threads; /* threads per interp block: 128, 256 or 512 */
    int32_t interp_coil_group; /* coils per interp thread block: 1, 2, 4 or 8 (0: the
                                  group that pads the coil count least) */
    int32_t interp_staging;    /* 2-D interp windows and 3-D interp planes: 0 = tensor-
                                  memory-access copies where the grid allows (default),
                                  1 = thread loads */
    int32_t dense_tile_samples; /* 3-D spread: tiles with at least this many samples (the
                                   k-space centre of radial data) accumulate with Kahan-
                                   compensated FP32 sums; 0 = 32768, negative = never */
    int32_t spread_variant;     /* spread with 8 coils per block: 0 = library choice
                                   (tensor cores on the default 4 x 8 x 16 tile, warp rows
                                   on a caller's tile), 1 = warp rows (tile (4 x warps / TY, TY, 16)),
                                   2 = 4^3-cell cubes fed by producer warps (tile of 8 or 16
                                   cubes; default work items of 2048 samples),
                                   3 = tensor cores (tcgen05 TF32 MMAs, 3-term split; tile
                                   4 x 8 x 16, default work items of 4096 samples, dense
                                   items on a compensated instance; in 2-D
                                   tile 8 x 16, selectable, slower than the 2-D default) */
    int32_t interp_variant;     /* 3-D interp with 8 coils per group: 0 = library choice (tensor
                                   cores whenever the spread's tiles are the tensor-core
                                   kernel's 4 x 8 x 16), 1 = the plane-streaming / window
                                   kernels on the interp's own bins, 2 = tensor cores where
                                   the spread's tiles allow (per tile a TF32 GEMM over the
                                   tile's samples, partial sums added with float atomics) */
    int32_t fft_variant;        /* FFT of the composite calls (type 1/2/21, SENSE): 0 = library
                                   choice (pruned on 3-D grids of >= 2^21 cells per instance,
                                   <= 256 instances; the full transform if cuFFT cannot make
                                   the pruned plans), 1 = the full transform, 2 = pruned
                                   wherever the image band is narrower than the grid (2-D and
                                   3-D, <= 4096 instances).  Pruned: the trailing axes are
                                   transformed only on the grid planes inside the image band
                                   along x, which hold every non-zero cell of the pad and
                                   every cell the crop reads (see gbn_fft_band) */
} gbn_plan_desc;

typedef struct {
    int32_t nspread;        /* half-width: 2*nspread taps per dimension */
    int32_t nf[3];          /* oversampled grid per dim (1 beyond dim) */
    double tau;             /* Gaussian g(x) = exp(-x^2 / (4 tau)) */
    int64_t n_samples;      /* total samples over all trajectory groups */
    int64_t grid_cells;     /* nf1*nf2*nf3 */
    int64_t n_inst;         /* n_traj * n_coil */
    int64_t spread_subproblems;
    int64_t interp_subproblems;
    int64_t spread_entries; /* (sample, tile) pairs in the spread lists */
    int32_t spread_tile[3];
    int32_t interp_tile[3];
    int32_t coil_group;
    int32_t threads;
    int32_t interp_threads;
    int32_t max_subproblem;
    int64_t device_bytes;   /* device memory held by the plan */
    int32_t interp_coil_group;
    int64_t dense_subproblems; /* spread subproblems with compensated accumulation */
    int32_t spread_kernels;    /* kernels the plan's last spread launched (0 before one) */
    int64_t split_tiles;       /* spread tiles shared by several work items (float atomics; 0 means
                                  the spread is bitwise reproducible run to run) */
    int32_t spread_variant;    /* the spread kernel this plan runs with 8 coils per block: 3 tensor
                                  cores (2-D or 3-D); in 3-D 1 warp rows, 2 cubes; 0 others */
    int32_t interp_variant;    /* 2 when the interp runs on the tensor cores (3-D, 8 coils per
                                  group; partial sums added with float atomics, so the
                                  samples agree run to run to rounding), else 1 */
    int32_t fft_variant;       /* 2 when the composite calls run the pruned transform, else 1 */
} gbn_plan_info;

/* element strides (in complex64 elements) of a strided complex array */
typedef struct {
    int64_t traj_stride;    /* between trajectory groups (images only) */
    int64_t coil_stride;    /* between coils */
    int64_t elem_stride;    /* between pixels (row-major pixel index) or samples */
} gbn_layout;

/* ---- library ------------------------------------------------------------ */
int gbn_version(void);
const char *gbn_status_string(int status);
/* copies the calling thread's last error message into buf (NUL-terminated) */
int gbn_last_error(char *buf, int len);

/* nspread, nf, tau from eps exactly as _compute_{1,2,3}d_grid_params
 * (fft/nufft_func.py:198-249); max_nspread > 0 applies the 3-D clamp to [3, max]. */
int gbn_grid_params(int dim, int ms, int mt, int mu, double eps, int max_nspread, int *nspread,
                    int64_t nf[3], double *tau);

/* ---- plans (replace the per-call set-up inside nufft{1,2,3}d{1,2,21}_gaussker) */
int gbn_plan_create(const gbn_plan_desc *desc, gbn_plan **out);
int gbn_plan_destroy(gbn_plan *plan);
int gbn_plan_get_info(const gbn_plan *plan, gbn_plan_info *out);
/* Synchronises the stream and reads the plan's device status word: GBN_ERR_TIMEOUT if a
 * kernel's bounded wait (the tensor copies of the 2-D interp windows and of the 3-D interp
 * planes) gave up since the last call, which also clears it; else GBN_OK.  No counterpart
 * in the reference (its kernels have no waits). */
int gbn_plan_status(gbn_plan *plan, gbn_stream_t stream);
/* Self-test of the path above, no counterpart in the reference: one thread arms an mbarrier
 * for 16 bytes that never arrive (no copy is issued, so nothing is in flight), waits with
 * the interp kernels' bounded wait cut to `probes` probes (1 .. 65536, each suspending at
 * most ~1 us) and, when the wait gives up, sets the status bit those kernels set.  The next
 * gbn_plan_status then returns GBN_ERR_TIMEOUT and clears it. */
int gbn_plan_check_wait_expiry(gbn_plan *plan, uint32_t probes, gbn_stream_t stream);

/* Sorts the samples into spatial bins (device coordinates, float32 or float64,
 * x/y/z each of length traj_offsets[n_traj]; unused dims may be NULL).
 * traj_offsets is a HOST array of n_traj+1 prefix offsets.  Allocates and
 * synchronises the stream once; call before capturing a graph. */
int gbn_set_points(gbn_plan *plan, int coord_dtype, const void *x, const void *y, const void *z,
                   const int64_t *traj_offsets, gbn_stream_t stream);

/* the plan's own oversampled grid buffer, (n_inst, nf1, nf2, nf3) complex64 (device) */
void *gbn_plan_grid(gbn_plan *plan);

/* ---- stages ------------------------------------------------------------- */
/* spread: grid[inst] = sum_j c_j g(x_j - h m), output-stationary tiles
 * (build_grid_{2,3}d1_fast, fft/nufft_func.py:550-582, 863-911).  Every cell of
 * the grid is written.  c: device samples with layout (coil_stride, elem_stride);
 * the sample index is global over trajectory groups. */
int gbn_spread(gbn_plan *plan, const void *c, gbn_layout c_layout, void *grid, gbn_stream_t stream);

/* interp: c_j = w_j * sum_m grid[m] g(x_j - h m) (build_grid_{2,3}d2_fast,
 * nufft_func.py:607-639, 985-1032) WITHOUT the reference's 1/N, which
 * gbn_pad_deapod folds in; weight (device float per sample) may be NULL. */
int gbn_interp(gbn_plan *plan, const void *grid, void *c, gbn_layout c_layout, const float *weight,
               gbn_stream_t stream);

/* batched in-place C2C FFT of the grid over all instances (cuFFT). */
int gbn_fft(gbn_plan *plan, void *grid, int direction, gbn_stream_t stream);
/* The transform the composite calls run between the pad and the interp (band =
 * GBN_BAND_INPUT) and between the spread and the crop (GBN_BAND_OUTPUT).  With the plan's
 * pruned transform (gbn_plan_info.fft_variant 2) the trailing axes are transformed only on the
 * grid planes inside the image band along x, x in [0, m - m/2) and [nf - m/2, nf):
 * GBN_BAND_INPUT assumes every other plane is zero and gives the full transform;
 * GBN_BAND_OUTPUT leaves the cells of the other planes holding the x pass only.  Otherwise
 * it is gbn_fft.  No counterpart in the reference (numpy / cuFFT full transforms,
 * fft/nufft_func.py:751-764, fft/nufft_func_cuda.py). */
int gbn_fft_band(gbn_plan *plan, void *grid, int direction, int band, gbn_stream_t stream);

/* image -> zero-padded grid with (pi/tau)^(d/2) exp(tau|k|^2) / N
 * (nufft_func.py:751-764) */
int gbn_pad_deapod(gbn_plan *plan, const void *img, gbn_layout img_layout, void *grid,
                   gbn_stream_t stream);
/* grid -> image with (1/M) (pi/tau)^(d/2) exp(tau|k|^2) / N (nufft_func.py:728-738) */
int gbn_crop_deapod(gbn_plan *plan, const void *grid, void *img, gbn_layout img_layout,
                    gbn_stream_t stream);

/* ---- whole transforms (device buffers) ------------------------------------ */
/* type-1: nufft{1,2,3}d1_gaussker (nufft_func.py:438, 702, 1167; _cuda twins
 * nufft_func_cuda.py:581, 1463).  weight (device float per sample, may be NULL)
 * multiplies the samples first: NUFFT3d.backward's density_weighting
 * (pics/operators_class.py:341-349) fused into the spread. */
int gbn_type1(gbn_plan *plan, const void *c, gbn_layout c_layout, const float *weight, void *img,
              gbn_layout img_layout, gbn_stream_t stream);
/* type-2: nufft{1,2,3}d2_gaussker (nufft_func.py:470, 741, 1209; nufft_func_cuda.py:609, 1512) */
int gbn_type2(gbn_plan *plan, const void *img, gbn_layout img_layout, void *c, gbn_layout c_layout,
              gbn_stream_t stream);
/* type-21: nufft{1,2,3}d21_gaussker (nufft_func.py:506, 780, 1261; nufft_func_cuda.py:639, 1562);
 * dcf (device float per sample) may be NULL. */
int gbn_type21(gbn_plan *plan, const void *img, gbn_layout img_layout, void *out,
               gbn_layout out_layout, const float *dcf, gbn_stream_t stream);

/* ---- SENSE-fused operators (joint2operators(espirit, NUFFT), pics/operators_class.py:437-514) */
/* kdata[coil] = A (S_coil . x); x: one image per trajectory group; sens: (n_coil, pixels) */
int gbn_sense_forward(gbn_plan *plan, const void *x, gbn_layout x_layout, const void *sens,
                      gbn_layout sens_layout, void *kdata, gbn_layout k_layout, gbn_stream_t stream);
/* x = sum_coil conj(S_coil) . type1(dcf . kdata[coil]); dcf may be NULL */
int gbn_sense_adjoint(gbn_plan *plan, const void *kdata, gbn_layout k_layout, const float *dcf,
                      const void *sens, gbn_layout sens_layout, void *x, gbn_layout x_layout,
                      gbn_stream_t stream);
/* x_out = S^H type21(S x) with dcf (may be NULL): the CG-SENSE / FISTA normal operator */
int gbn_sense_normal(gbn_plan *plan, const void *x, gbn_layout x_layout, const void *sens,
                     gbn_layout sens_layout, const float *dcf, void *x_out, gbn_layout out_layout,
                     gbn_stream_t stream);

/* ---- differentiation ------------------------------------------------------ */
/* grad_xyz[j*dim + d] = df * Re( sum_coil conj(grad_c[j,coil]) dc_j/dx_{j,d} ) for c = interp(grid)
 * with the analytic derivative of the Gaussian weights (device float (M, dim)). */
int gbn_interp_grad_coords(gbn_plan *plan, const void *grid, const void *grad_c, gbn_layout c_layout,
                           float *grad_xyz, gbn_stream_t stream);

/* ---- CUDA graphs ------------------------------------------------------------ */
/* Captures gbn_sense_normal (sens != NULL) or gbn_type21 (sens == NULL) with fixed
 * pointers into a graph; replay with gbn_graph_launch on any stream. */
int gbn_graph_capture_normal(gbn_plan *plan, const void *x, gbn_layout x_layout, const void *sens,
                             gbn_layout sens_layout, const float *dcf, void *x_out,
                             gbn_layout out_layout, gbn_graph **out);
int gbn_graph_launch(gbn_graph *graph, gbn_stream_t stream);
int gbn_graph_destroy(gbn_graph *graph);

/* ---- solvers on the normal operator (pics/CS_MRI_solvers_func.py, pics/proximal_func.py) ---- */
/* Vectors (x, rhs): with sens, one image per trajectory group, (n_traj, pixels); without,
 * the plan's coil-last images (n_traj, pixels, n_coil); contiguous complex64, device.  The
 * normal operator N is gbn_sense_normal (sens != NULL) or gbn_type21 (sens == NULL) with
 * dcf (may be NULL).  Each iteration (operator + vector kernels) is one CUDA graph, captured
 * on the first call and replayed while the operator inputs, the workspace and the points
 * stay the same; all scalars stay in device memory, so the host never waits.  The plan
 * allocates its solver workspace (5 vectors) on first use.  Calls on one plan must not
 * overlap. */
#define GBN_SOLVE_X0 1        /* x holds the initial guess (else the solve starts from 0) */
#define GBN_SOLVE_NO_GRAPH 2  /* launch every kernel directly instead of replaying a graph */
#define GBN_SOLVE_FISTA 4     /* gbn_ista_haar: FISTA (FIST_32) instead of IST (IST_32) */
/* Linear CG on N x = rhs, n_iter iterations: the reference has no CG-SENSE routine (its
 * linear CG on the normal equations, pics/proximal_func.py:379-406, is commented out), so
 * this is that algorithm with forward_backward as N.  Inner products in FP64; res_norms
 * (device double[n_iter], may be NULL) receives ||r|| after every iteration.  With several
 * trajectory groups N is block-diagonal and the CG runs on all groups' images as one
 * vector (one set of scalars), not one CG per group. */
int gbn_cg_sense(gbn_plan *plan, const void *sens, gbn_layout sens_layout, const float *dcf,
                 const void *rhs, void *x, int32_t n_iter, double *res_norms, int32_t flags,
                 gbn_stream_t stream);
/* IST_32 (CS_MRI_solvers_func.py:75-86) or FIST_32 (:207-224) with rhs = A^H b (the
 * solvers' invAb), the transform T = level-`level` orthonormal Haar over the spatial axes
 * (DWTnd('haar'), pics/operators_class.py:394-416; level 0 = identity: IST_22 / FIST_22) and
 * prox_l1_Tf_soft_thresh2 (proximal_func.py:46-52).  Every image axis must be a multiple
 * of 2^level and dim * level <= 12.  x receives the final iterate. */
int gbn_ista_haar(gbn_plan *plan, const void *sens, gbn_layout sens_layout, const float *dcf,
                  const void *rhs, void *x, int32_t n_iter, float step, float th, int32_t level,
                  int32_t flags, gbn_stream_t stream);

/* Density compensation by Pipe-Menon iteration (J. G. Pipe, P. Menon, MRM 41:179, 1999):
 * w = 1, then n_iter times w <- w / |C w| with C w = interp(spread(w)) on the plan's own
 * Gaussian kernel and grid (no FFT); dcf (device float[M_total]) receives w scaled to mean
 * 1 in every trajectory group, so the normal operator's diagonal ((1/M) sum_j dcf_j) stays
 * 1 as without dcf.  The reference reads its dcf from files (examples/
 * pics_IST_3dute_wavelet_L1.py:31); this computes one for a trajectory.  The plan must have
 * n_coil == 1.  Uses the plan's grid. */
int gbn_dcf_pipe_menon(gbn_plan *plan, int32_t n_iter, float *dcf, gbn_stream_t stream);

/* ---- ESPIRiT coil maps (espirit/espirit_func.py) ---------------------------------- */
/* The pixel-wise eigen step of espirit_2d / espirit_3d (espirit_func.py:72-81, 186-196):
 * a (device, complex64, (n_pix, nsv, nc)) holds each pixel's nsv image-space ESPIRiT
 * kernels; for vvH = A^T conj(A) (nc x nc) the largest eigenvalue goes to smap (device
 * float[n_pix]) and its unit eigenvector to vmap (device complex64 (n_pix, nc)), by n_iter
 * power iterations from the column of the largest diagonal entry.  The reference takes the
 * SVD of vvH, whose eigenvector phase is arbitrary per pixel; here coil 0's component (the
 * first non-zero coil's) is real and non-negative.  nc <= 32. */
int gbn_espirit_eigen(const void *a, int64_t n_pix, int32_t nsv, int32_t nc, int32_t n_iter, void *vmap,
                      float *smap, gbn_stream_t stream);

/* ---- wavelet and proximal operators (no plan) ------------------------------------- */
/* Orthonormal level-`level` Haar transform of complex64 arrays (n_outer, s0[, s1[, s2]],
 * n_inner) over the dim spatial axes (contiguous, device): DWTnd('haar', level, axes)
 * .backward (image -> coefficients, inverse = 0) and .forward (inverse = 1), pics/
 * operators_class.py:394-416, coefficients in the layout of pywt.coeffs_to_array
 * (approximation block first along every axis, then each level's detail blocks, coarsest
 * first).  in and out must differ.  Axis sizes multiples of 2^level; dim * level <= 12. */
int gbn_haar_dwt(int32_t dim, const int32_t *shape, int32_t level, int64_t n_outer, int64_t n_inner,
                 const void *in, void *out, int32_t inverse, gbn_stream_t stream);
/* out = H^-1 soft(H in, th) with H the Haar transform above and soft the reference's
 * prox_l1_soft_thresh2 (proximal_func.py:20-24): v / (|v| + 1e-6) * max(|v| - th, 0);
 * prox_l1_Tf_soft_thresh2 (:46-52) with DWTnd('haar').  in == out allowed. */
int gbn_prox_haar(int32_t dim, const int32_t *shape, int32_t level, int64_t n_outer, int64_t n_inner,
                  const void *in, float th, void *out, gbn_stream_t stream);

/* ---- allocation-free spread ------------------------------------------------------------ */
/* No counterpart in the reference.  The 2-D spread of gbn_spread (samples -> oversampled
 * grid, (n_coil, nf1, nf2) complex64, nf from eps as gbn_grid_params) for callers that
 * cannot allocate device memory: code inside a framework that owns the GPU memory pool,
 * real-time loops that must not block in cudaMalloc, plugin hosts that pass only pre-sized
 * buffers.  The caller passes device inputs and the output grid; the binning scratch is a
 * fixed file-scope device array (about 8.7 MiB, held by every GPU that loads the library),
 * so nothing is allocated.  Limits: M <= GBN_NOALLOC_MAX_SAMPLES, nspread <= 8, ms % 8 == 0,
 * mt % 16 == 0, grid of at most GBN_NOALLOC_MAX_TILES 16x32 tiles (else GBN_ERR_CAPACITY).
 * All calls share the array: calls that overlap on the GPU race, so order them on one
 * stream.  The first call on a device resolves the array's address and, under CUDA's lazy
 * module loading, is where the driver commits the array's memory on that device (so it can
 * fail with GBN_ERR_CUDA when the device is full): make it during set-up, before any stream
 * capture.  The address is kept for the device's primary context; after cudaDeviceReset,
 * or from a different driver context, it is stale.  A sample with a non-finite coordinate
 * is left out (it adds nothing to the grid; the plan path reports it as an error instead). */
#define GBN_NOALLOC_MAX_SAMPLES 262144
#define GBN_NOALLOC_MAX_TILES 16384
int gbn_spread2d_noalloc(int coord_dtype, const void *x, const void *y, int64_t M, const void *c,
                         gbn_layout c_layout, int32_t n_coil, int32_t ms, int32_t mt, double eps, double df,
                         void *grid, gbn_stream_t stream);

/* ---- host-buffer entry points (the reference's numpy-in / numpy-out calls) ---- */
/* One call = inputs from host memory, the transform, the result into host memory,
 * synchronised.  Pageable arrays go through the plan's staging buffers (H2D copy,
 * transform, D2H copy).  Pinned (page-locked) arrays are read and written by the
 * kernels directly over the host link where the access pattern allows (image in the
 * pad, samples out of the interp, image out of the crop), which overlaps the transfer
 * with the compute; the samples of type-1 are always copied in bulk (the spread reads
 * each several times).  Layouts are the reference's: image (ms, mt[, mu], n_coil)
 * coil-last per trajectory group, samples (M_total, n_coil) coil-last; complex64. */
int gbn_type1_host(gbn_plan *plan, const void *h_c, void *h_img, gbn_stream_t stream);
int gbn_type2_host(gbn_plan *plan, const void *h_img, void *h_c, gbn_stream_t stream);
int gbn_type21_host(gbn_plan *plan, const void *h_img, void *h_out, const float *h_dcf,
                    gbn_stream_t stream);

/* One-shot calls with the reference's signatures (host float64 coordinates,
 * complex64 data coil-last, ntrail coils): plan, sort, transform, free.
 * nufft2d1_gaussker fft/nufft_func.py:702 / nufft_func_cuda.py:581 */
int gbn_nufft2d1_gaussker(const double *x, const double *y, const void *c, int64_t M, int32_t ntrail,
                          int32_t ms, int32_t mt, double df, double eps, int32_t iflag, void *out);
/* nufft2d2_gaussker fft/nufft_func.py:741 / nufft_func_cuda.py:609 */
int gbn_nufft2d2_gaussker(const double *x, const double *y, const void *Fk, int64_t M, int32_t ntrail,
                          int32_t ms, int32_t mt, double df, double eps, int32_t iflag, void *out);
/* nufft2d21_gaussker fft/nufft_func.py:780 / nufft_func_cuda.py:639 */
int gbn_nufft2d21_gaussker(const double *x, const double *y, const void *Fk, int64_t M, int32_t ntrail,
                           int32_t ms, int32_t mt, double df, double eps, int32_t iflag, void *out);
/* nufft3d1_gaussker fft/nufft_func.py:1167 / nufft_func_cuda.py:1463 */
int gbn_nufft3d1_gaussker(const double *x, const double *y, const double *z, const void *c, int64_t M,
                          int32_t ntrail, int32_t ms, int32_t mt, int32_t mu, double df, double eps,
                          int32_t iflag, void *out);
/* nufft3d2_gaussker fft/nufft_func.py:1209 / nufft_func_cuda.py:1512 */
int gbn_nufft3d2_gaussker(const double *x, const double *y, const double *z, const void *Fk, int64_t M,
                          int32_t ntrail, int32_t ms, int32_t mt, int32_t mu, double df, double eps,
                          int32_t iflag, void *out);
/* nufft3d21_gaussker fft/nufft_func.py:1261 / nufft_func_cuda.py:1562 (dcf may be NULL) */
int gbn_nufft3d21_gaussker(const double *x, const double *y, const double *z, const void *Fk,
                           int64_t M, int32_t ntrail, int32_t ms, int32_t mt, int32_t mu,
                           const double *dcf, double df, double eps, int32_t iflag, void *out);

#ifdef __cplusplus
}
#endif
#endif /* GBNUFFT_H */
