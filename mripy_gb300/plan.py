"""``NufftPlan``: a GPU NUFFT plan over the C ABI, driven with PyTorch CUDA tensors.

A plan fixes the image shape, accuracy (eps -> nspread, oversampled grid, tau, as in
mripy's ``_compute_{1,2,3}d_grid_params``, fft/nufft_func.py:198-249), the number of
coils sharing each trajectory and the number of trajectory groups (frames or slices
with their own, ragged, sample counts).  ``set_points`` bins the samples once; every
transform afterwards is a stream-ordered sequence of kernel launches with no host
synchronisation, so it can be captured in a CUDA graph.

Canonical tensor shapes (complex64, CUDA, any strides as long as the image axes are
mutually contiguous):
  images   (n_traj, *shape, n_coil)
  samples  (M_total, n_coil)        sample index global over the trajectory groups
  coil maps (*shape, n_coil)        (SENSE operators)
  SENSE images (n_traj, *shape)
"""
import ctypes

import torch

from . import _native as N


def grid_params(dim, ms, mt=1, mu=1, eps=1e-15, max_nspread=0):
    """(nspread, (nf1, nf2, nf3), tau) exactly as the reference chooses them."""
    ns = ctypes.c_int32()
    nf = (ctypes.c_int64 * 3)()
    tau = ctypes.c_double()
    N.check(N.lib().gbn_grid_params(dim, ms, mt, mu, float(eps), int(max_nspread or 0), ctypes.byref(ns), nf,
                                    ctypes.byref(tau)))
    return ns.value, tuple(nf[:dim]), tau.value


_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)


def _stream(stream=None):
    """The cudaStream_t of ``stream``, else of torch's current stream (read without building a
    Stream object: that costs ~20 us a call, several times per transform)."""
    if stream is not None:
        return ctypes.c_void_p(stream.cuda_stream)
    if _raw_stream is not None:
        return ctypes.c_void_p(_raw_stream(torch.cuda.current_device()))
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _require_cuda(t, name, dtype=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if dtype is not None and t.dtype != dtype:
        raise TypeError("%s must be %s, got %s" % (name, dtype, t.dtype))


class Tuning:
    """Kernel tiling chosen by the autotuner (0 = library default)."""

    def __init__(self, spread_tile=(0, 0, 0), interp_tile=(0, 0, 0), max_subproblem=0, coil_group=0, threads=0,
                 interp_threads=0, interp_coil_group=0, interp_staging=0, spread_variant=0, interp_variant=0,
                 fft_variant=0):
        self.spread_tile = tuple(spread_tile) + (0,) * (3 - len(spread_tile))
        self.interp_tile = tuple(interp_tile) + (0,) * (3 - len(interp_tile))
        self.max_subproblem = max_subproblem
        self.coil_group = coil_group
        self.threads = threads
        self.interp_threads = interp_threads
        self.interp_coil_group = interp_coil_group
        self.interp_staging = interp_staging  # 0 tensor copies (TMA) where possible, 1 thread loads
        self.spread_variant = spread_variant  # 3-D, 8 coils: 0 library choice, 1 warp rows, 2 cubes, 3 tensor cores
        self.interp_variant = interp_variant  # 3-D, 8 coils: 0 library choice, 1 plane streaming, 2 tensor cores
        self.fft_variant = fft_variant  # composite calls' FFT: 0 library choice, 1 full, 2 pruned to the image band

    def key(self):
        return (self.spread_tile, self.interp_tile, self.max_subproblem, self.coil_group, self.threads,
                self.interp_threads, self.interp_coil_group, self.interp_staging, self.spread_variant,
                self.interp_variant, self.fft_variant)

    def __repr__(self):
        return ("Tuning(spread_tile=%s, interp_tile=%s, max_subproblem=%d, coil_group=%d, threads=%d, "
                "interp_threads=%d, interp_coil_group=%d, interp_staging=%d, spread_variant=%d, "
                "interp_variant=%d, fft_variant=%d)" % (
                    self.spread_tile, self.interp_tile, self.max_subproblem, self.coil_group, self.threads,
                    self.interp_threads, self.interp_coil_group, self.interp_staging, self.spread_variant,
                    self.interp_variant, self.fft_variant))


class Graph:
    """A captured normal operator; ``launch()`` replays it on the current stream."""

    def __init__(self, handle, keep):
        self._h = handle
        self._keep = keep  # tensors whose pointers the graph holds

    def launch(self, stream=None):
        N.check(N.lib().gbn_graph_launch(self._h, _stream(stream)))

    def close(self):
        if self._h:
            N.lib().gbn_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NufftPlan:
    def __init__(self, dim, shape, n_coil=1, n_traj=1, eps=1e-15, iflag=1, df=1.0, max_nspread=None,
                 tuning=None, dense_tile_samples=0):
        """dense_tile_samples (3-D): spread tiles with at least this many samples accumulate
        with Kahan-compensated FP32 sums; 0 = library default (32768), negative = never."""
        shape = tuple(int(s) for s in shape)
        if len(shape) != dim:
            raise ValueError("shape must have %d entries" % dim)
        self.dim = dim
        self.shape = shape
        self.n_coil = int(n_coil)
        self.n_traj = int(n_traj)
        self.eps = float(eps)
        self.iflag = int(iflag)
        self.df = float(df)
        self.tuning = tuning or Tuning()
        d = N.PlanDesc()
        d.dim = dim
        d.ms = shape[0]
        d.mt = shape[1] if dim > 1 else 1
        d.mu = shape[2] if dim > 2 else 1
        d.eps = self.eps
        d.max_nspread = int(max_nspread or 0)
        d.iflag = self.iflag
        d.df = self.df
        d.n_coil = self.n_coil
        d.n_traj = self.n_traj
        for i in range(3):
            d.spread_tile[i] = int(self.tuning.spread_tile[i])
            d.interp_tile[i] = int(self.tuning.interp_tile[i])
        d.max_subproblem = int(self.tuning.max_subproblem)
        d.coil_group = int(self.tuning.coil_group)
        d.threads = int(self.tuning.threads)
        d.interp_threads = int(self.tuning.interp_threads)
        d.interp_coil_group = int(self.tuning.interp_coil_group)
        d.interp_staging = int(self.tuning.interp_staging)
        d.dense_tile_samples = int(dense_tile_samples)
        d.spread_variant = int(getattr(self.tuning, "spread_variant", 0))
        d.interp_variant = int(getattr(self.tuning, "interp_variant", 0))
        d.fft_variant = int(getattr(self.tuning, "fft_variant", 0))
        self._lib = N.lib()
        h = ctypes.c_void_p()
        N.check(self._lib.gbn_plan_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self.traj_offsets = None
        self.n_samples = 0
        self.points_generation = 0  # bumped by every set_points

    # ------------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._lib.gbn_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        inf = N.PlanInfo()
        N.check(self._lib.gbn_plan_get_info(self._h, ctypes.byref(inf)))
        return {
            "nspread": inf.nspread, "nf": tuple(inf.nf[:self.dim]), "tau": inf.tau,
            "n_samples": inf.n_samples, "grid_cells": inf.grid_cells, "n_inst": inf.n_inst,
            "spread_subproblems": inf.spread_subproblems, "interp_subproblems": inf.interp_subproblems,
            "spread_entries": inf.spread_entries, "spread_tile": tuple(inf.spread_tile[:self.dim]),
            "interp_tile": tuple(inf.interp_tile[:self.dim]), "coil_group": inf.coil_group,
            "threads": inf.threads, "interp_threads": inf.interp_threads, "max_subproblem": inf.max_subproblem,
            "device_bytes": inf.device_bytes, "interp_coil_group": inf.interp_coil_group,
            "dense_subproblems": inf.dense_subproblems,
            "spread_kernels": inf.spread_kernels, "split_tiles": inf.split_tiles,
            "spread_variant": inf.spread_variant, "interp_variant": inf.interp_variant,
            "fft_variant": inf.fft_variant,
        }

    def status(self, stream=None):
        """Synchronise and raise GbnError(GBN_ERR_TIMEOUT) if a kernel's bounded wait gave up."""
        N.check(self._lib.gbn_plan_status(self._h, _stream(stream)))

    def check_wait_expiry(self, probes=64, stream=None):
        """Self-test of the bounded-wait status path: a one-thread kernel waits for bytes that
        never arrive, gives up after ``probes`` probes and sets the plan's timeout bit (read
        and cleared by ``status()``)."""
        N.check(self._lib.gbn_plan_check_wait_expiry(self._h, int(probes), _stream(stream)))

    def grid(self):
        """The plan's oversampled grid buffer as a (n_traj*n_coil, *nf) complex64 view."""
        inf = self.info()
        ptr = self._lib.gbn_plan_grid(self._h)
        n = inf["n_inst"] * inf["grid_cells"]
        return _from_ptr(ptr, n).view((inf["n_inst"],) + inf["nf"])

    # ------------------------------------------------------------------ points
    def set_points(self, coords, traj_offsets=None, stream=None):
        """coords: ``dim`` CUDA tensors (float32 or float64) of length M_total, radians.
        traj_offsets: n_traj+1 prefix offsets (host ints); default one group."""
        if len(coords) != self.dim:
            raise ValueError("need %d coordinate arrays" % self.dim)
        dt = coords[0].dtype
        if dt not in (torch.float32, torch.float64):
            raise TypeError("coordinates must be float32 or float64")
        M = coords[0].numel()
        cs = []
        for c in coords:
            _require_cuda(c, "coordinate", dt)
            if c.numel() != M:
                raise ValueError("coordinate arrays differ in length")
            cs.append(c.contiguous().view(-1))
        if traj_offsets is None:
            traj_offsets = [0, M]
        off = [int(v) for v in traj_offsets]
        if len(off) != self.n_traj + 1 or off[-1] != M:
            raise ValueError("traj_offsets must have n_traj+1 entries ending at M")
        arr = (ctypes.c_int64 * len(off))(*off)
        ptrs = [_ptr(c) for c in cs] + [None] * (3 - self.dim)
        N.check(self._lib.gbn_set_points(self._h, N.GBN_COORD_F64 if dt == torch.float64 else N.GBN_COORD_F32,
                                         ptrs[0], ptrs[1], ptrs[2], arr, _stream(stream)))
        self.traj_offsets = off
        self.n_samples = M
        self.points_generation += 1
        return self

    # ------------------------------------------------------------------ layouts
    def _img_layout(self, t, name="image"):
        _require_cuda(t, name, torch.complex64)
        want = (self.n_traj,) + self.shape + (self.n_coil,)
        if tuple(t.shape) != want:
            raise ValueError("%s must have shape %s, got %s" % (name, want, tuple(t.shape)))
        st = t.stride()
        for d in range(1, self.dim):
            if st[d] != st[d + 1] * t.shape[d + 1]:
                raise ValueError("%s image axes must be mutually contiguous" % name)
        return N.Layout(st[0], st[-1], st[self.dim])

    def _sample_layout(self, t, name="samples"):
        _require_cuda(t, name, torch.complex64)
        want = (self.n_samples, self.n_coil)
        if tuple(t.shape) != want:
            raise ValueError("%s must have shape %s, got %s" % (name, want, tuple(t.shape)))
        st = t.stride()
        return N.Layout(0, st[1], st[0])

    def _sense_layout(self, s):
        _require_cuda(s, "coil maps", torch.complex64)
        want = self.shape + (self.n_coil,)
        if tuple(s.shape) != want:
            raise ValueError("coil maps must have shape %s, got %s" % (want, tuple(s.shape)))
        st = s.stride()
        for d in range(0, self.dim - 1):
            if st[d] != st[d + 1] * s.shape[d + 1]:
                raise ValueError("coil-map image axes must be mutually contiguous")
        return N.Layout(0, st[-1], st[self.dim - 1])

    def _x_layout(self, x, name="x"):
        _require_cuda(x, name, torch.complex64)
        want = (self.n_traj,) + self.shape
        if tuple(x.shape) != want:
            raise ValueError("%s must have shape %s, got %s" % (name, want, tuple(x.shape)))
        st = x.stride()
        for d in range(1, self.dim):
            if st[d] != st[d + 1] * x.shape[d + 1]:
                raise ValueError("%s image axes must be mutually contiguous" % name)
        return N.Layout(st[0], 0, st[self.dim])

    @staticmethod
    def _weight(w, M):
        if w is None:
            return None
        _require_cuda(w, "dcf", torch.float32)
        if w.numel() != M or not w.is_contiguous():
            raise ValueError("dcf must be a contiguous float32 vector of length M_total")
        return _ptr(w)

    def _check_points(self):
        if self.traj_offsets is None:
            raise N.GbnError(5, "set_points has not been called")

    def empty_image(self):
        return torch.empty((self.n_traj,) + self.shape + (self.n_coil,), dtype=torch.complex64, device="cuda")

    def empty_samples(self):
        return torch.empty((self.n_samples, self.n_coil), dtype=torch.complex64, device="cuda")

    # ------------------------------------------------------------------ transforms
    def type1(self, c, out=None, weight=None, stream=None):
        """(1/M_g) sum_j w_j c_j exp(+s i k.x_j) per group and coil (nufft{1,2,3}d1_gaussker;
        the optional per-sample weight is the operators' density compensation)."""
        self._check_points()
        out = self.empty_image() if out is None else out
        N.check(self._lib.gbn_type1(self._h, _ptr(c), self._sample_layout(c), self._weight(weight, self.n_samples),
                                    _ptr(out), self._img_layout(out), _stream(stream)))
        return out

    def type2(self, img, out=None, stream=None):
        """sum_k F_k exp(-s i k.x_j) (nufft{1,2,3}d2_gaussker)."""
        self._check_points()
        out = self.empty_samples() if out is None else out
        N.check(self._lib.gbn_type2(self._h, _ptr(img), self._img_layout(img), _ptr(out),
                                    self._sample_layout(out), _stream(stream)))
        return out

    def type21(self, img, dcf=None, out=None, stream=None):
        """(1/M_g) A^H D A F (nufft{1,2,3}d21_gaussker)."""
        self._check_points()
        out = self.empty_image() if out is None else out
        N.check(self._lib.gbn_type21(self._h, _ptr(img), self._img_layout(img), _ptr(out),
                                     self._img_layout(out, "out"), self._weight(dcf, self.n_samples),
                                     _stream(stream)))
        return out

    def spread(self, c, grid=None, stream=None):
        self._check_points()
        grid = self.grid() if grid is None else grid
        N.check(self._lib.gbn_spread(self._h, _ptr(c), self._sample_layout(c), _ptr(grid), _stream(stream)))
        return grid

    def interp(self, grid, out=None, weight=None, stream=None):
        self._check_points()
        out = self.empty_samples() if out is None else out
        N.check(self._lib.gbn_interp(self._h, _ptr(grid), _ptr(out), self._sample_layout(out),
                                     self._weight(weight, self.n_samples), _stream(stream)))
        return out

    def fft(self, grid, direction, stream=None):
        N.check(self._lib.gbn_fft(self._h, _ptr(grid), int(direction), _stream(stream)))
        return grid

    def fft_band(self, grid, direction, band, stream=None):
        """The transform of the composite calls: ``band`` = ``GBN_BAND_INPUT`` after the pad
        (the grid is zero outside the image band along x), ``GBN_BAND_OUTPUT`` before the crop
        (only the band is read afterwards).  The full transform unless ``info()["fft_variant"]``
        is 2."""
        N.check(self._lib.gbn_fft_band(self._h, _ptr(grid), int(direction), int(band), _stream(stream)))
        return grid

    def pad_deapod(self, img, grid=None, stream=None):
        grid = self.grid() if grid is None else grid
        N.check(self._lib.gbn_pad_deapod(self._h, _ptr(img), self._img_layout(img), _ptr(grid), _stream(stream)))
        return grid

    def crop_deapod(self, grid, out=None, stream=None):
        self._check_points()
        out = self.empty_image() if out is None else out
        N.check(self._lib.gbn_crop_deapod(self._h, _ptr(grid), _ptr(out), self._img_layout(out), _stream(stream)))
        return out

    # ------------------------------------------------------------------ SENSE
    def sense_forward(self, x, sens, out=None, stream=None):
        self._check_points()
        out = self.empty_samples() if out is None else out
        N.check(self._lib.gbn_sense_forward(self._h, _ptr(x), self._x_layout(x), _ptr(sens), self._sense_layout(sens),
                                            _ptr(out), self._sample_layout(out), _stream(stream)))
        return out

    def sense_adjoint(self, kdata, sens, dcf=None, out=None, stream=None):
        self._check_points()
        out = torch.empty((self.n_traj,) + self.shape, dtype=torch.complex64, device="cuda") if out is None else out
        N.check(self._lib.gbn_sense_adjoint(self._h, _ptr(kdata), self._sample_layout(kdata),
                                            self._weight(dcf, self.n_samples), _ptr(sens), self._sense_layout(sens),
                                            _ptr(out), self._x_layout(out, "out"), _stream(stream)))
        return out

    def sense_normal(self, x, sens, dcf=None, out=None, stream=None):
        self._check_points()
        out = torch.empty((self.n_traj,) + self.shape, dtype=torch.complex64, device="cuda") if out is None else out
        N.check(self._lib.gbn_sense_normal(self._h, _ptr(x), self._x_layout(x), _ptr(sens), self._sense_layout(sens),
                                           self._weight(dcf, self.n_samples), _ptr(out), self._x_layout(out, "out"),
                                           _stream(stream)))
        return out

    # ------------------------------------------------------------------ solvers
    def _solve_vec(self, t, sens, name):
        want = (self.n_traj,) + self.shape + (() if sens is not None else (self.n_coil,))
        _require_cuda(t, name, torch.complex64)
        if tuple(t.shape) != want or not t.is_contiguous():
            raise ValueError("%s must be a contiguous complex64 tensor of shape %s, got %s"
                             % (name, want, tuple(t.shape)))

    def cg(self, rhs, n_iter, sens=None, dcf=None, x0=None, use_graph=True, stream=None):
        """Linear CG on N x = rhs with N = S^H type21(S .) (sens given; x, rhs: (n_traj,
        *shape)) or type21 (x, rhs: (n_traj, *shape, n_coil)).  Returns (x, residual norms
        after every iteration, float64 device tensor)."""
        self._check_points()
        self._solve_vec(rhs, sens, "rhs")
        if x0 is not None:
            self._solve_vec(x0, sens, "x0")
            x = x0.clone()
        else:
            x = torch.empty_like(rhs)
        norms = torch.empty(int(n_iter), dtype=torch.float64, device="cuda")
        sl = self._sense_layout(sens) if sens is not None else N.Layout(0, 0, 0)
        flags = (N.GBN_SOLVE_X0 if x0 is not None else 0) | (0 if use_graph else N.GBN_SOLVE_NO_GRAPH)
        N.check(self._lib.gbn_cg_sense(self._h, _ptr(sens), sl, self._weight(dcf, self.n_samples), _ptr(rhs),
                                       _ptr(x), int(n_iter), _ptr(norms), flags, _stream(stream)))
        return x, norms

    def ista(self, rhs, n_iter, step, th, level, sens=None, dcf=None, fista=True, use_graph=True, stream=None):
        """IST_32 / FIST_32 with rhs = A^H b and the level-``level`` Haar soft-threshold prox
        (level 0: plain soft threshold).  Vectors as in :meth:`cg`.  Returns x."""
        self._check_points()
        self._solve_vec(rhs, sens, "rhs")
        x = torch.empty_like(rhs)
        sl = self._sense_layout(sens) if sens is not None else N.Layout(0, 0, 0)
        flags = (N.GBN_SOLVE_FISTA if fista else 0) | (0 if use_graph else N.GBN_SOLVE_NO_GRAPH)
        N.check(self._lib.gbn_ista_haar(self._h, _ptr(sens), sl, self._weight(dcf, self.n_samples), _ptr(rhs),
                                        _ptr(x), int(n_iter), float(step), float(th), int(level), flags,
                                        _stream(stream)))
        return x

    def pipe_menon_dcf(self, n_iter=20, out=None, stream=None):
        """Density compensation of this plan's trajectory by Pipe-Menon iteration on the
        plan's Gaussian kernel: (M_total,) float32, mean 1 per trajectory group.  Needs a
        plan with n_coil == 1; overwrites the plan's grid."""
        self._check_points()
        out = torch.empty(self.n_samples, dtype=torch.float32, device="cuda") if out is None else out
        _require_cuda(out, "out", torch.float32)
        if out.numel() != self.n_samples or not out.is_contiguous():
            raise ValueError("out must be a contiguous float32 tensor of %d elements" % self.n_samples)
        N.check(self._lib.gbn_dcf_pipe_menon(self._h, int(n_iter), _ptr(out), _stream(stream)))
        return out

    # ------------------------------------------------------------------ gradient
    def interp_grad_coords(self, grid, grad_c, out=None, stream=None):
        """(M_total, dim) float32: df * Re(sum_coil conj(grad_c) dc/dx) for c = interp(grid)."""
        self._check_points()
        out = torch.empty((self.n_samples, self.dim), dtype=torch.float32, device="cuda") if out is None else out
        N.check(self._lib.gbn_interp_grad_coords(self._h, _ptr(grid), _ptr(grad_c), self._sample_layout(grad_c, "grad"),
                                                 _ptr(out), _stream(stream)))
        return out

    # ------------------------------------------------------------------ graphs
    def capture_normal(self, x, out, sens=None, dcf=None):
        """Capture the normal operator on fixed buffers: S^H type21(S x) when ``sens`` is
        given (x, out: (n_traj, *shape)), else type21 (x, out: canonical images)."""
        self._check_points()
        h = ctypes.c_void_p()
        if sens is not None:
            xl, ol, sl = self._x_layout(x), self._x_layout(out, "out"), self._sense_layout(sens)
        else:
            xl, ol, sl = self._img_layout(x), self._img_layout(out, "out"), N.Layout(0, 0, 0)
        N.check(self._lib.gbn_graph_capture_normal(self._h, _ptr(x), xl, _ptr(sens), sl,
                                                   self._weight(dcf, self.n_samples), _ptr(out), ol,
                                                   ctypes.byref(h)))
        return Graph(h, (x, out, sens, dcf, self))


def _haar_layout(x, axes):
    axes = tuple(int(a) % x.dim() for a in axes)
    d = len(axes)
    if d < 1 or d > 3 or axes != tuple(range(axes[0], axes[0] + d)):
        raise NotImplementedError("the Haar kernels take 1 to 3 consecutive, increasing axes, got %s" % (axes,))
    _require_cuda(x, "x", torch.complex64)
    if not x.is_contiguous():
        raise ValueError("x must be contiguous")
    outer, inner = 1, 1
    for s in x.shape[:axes[0]]:
        outer *= int(s)
    for s in x.shape[axes[0] + d:]:
        inner *= int(s)
    shape = (ctypes.c_int32 * 3)(*([int(x.shape[a]) for a in axes] + [1] * (3 - d)))
    return d, shape, outer, inner


def haar_dwt(x, level, axes, inverse=False, out=None, stream=None):
    """Orthonormal level-``level`` Haar transform over ``axes`` of a complex64 CUDA tensor:
    image -> coefficients in pywt.coeffs_to_array's layout (inverse=False), or back."""
    d, shape, outer, inner = _haar_layout(x, axes)
    out = torch.empty_like(x) if out is None else out
    if out.shape != x.shape or out.data_ptr() == x.data_ptr():
        raise ValueError("out must be a separate tensor of the input's shape")
    N.check(N.lib().gbn_haar_dwt(d, shape, int(level), outer, inner, _ptr(x), _ptr(out), 1 if inverse else 0,
                                 _stream(stream)))
    return out


def prox_haar(x, th, level, axes, out=None, stream=None):
    """H^-1 soft(H x, th) with the level-``level`` Haar transform over ``axes`` (level 0:
    the plain soft threshold x / (|x| + 1e-6) * max(|x| - th, 0))."""
    d, shape, outer, inner = _haar_layout(x, axes)
    out = torch.empty_like(x) if out is None else out
    N.check(N.lib().gbn_prox_haar(d, shape, int(level), outer, inner, _ptr(x), float(th), _ptr(out),
                                  _stream(stream)))
    return out


def _from_ptr(ptr, n):
    """Wrap a library-owned complex64 device buffer as a tensor (no copy, not owned)."""
    class _Holder:
        pass

    holder = _Holder()
    holder.__cuda_array_interface__ = {
        "shape": (2 * int(n),), "typestr": "<f4", "data": (int(ptr), False), "version": 3, "strides": None,
    }
    return torch.as_tensor(holder, device="cuda").view(torch.complex64)
