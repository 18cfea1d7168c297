"""NUFFT operator classes with the interface of mripy's ``NUFFT3d`` /
``NUFFT3d_cuda`` (pics/operators_class.py:302-364, pics/operators_cuda_class.py:64-127),
a 2-D ``NUFFT2d`` with the same interface, the coil-sensitivity operator ``espirit``
and ``joint2operators`` (pics/operators_class.py:437-514).

* ``forward(im)``           type-2 NUFFT, image (nx, ny[, nz][, nc]) -> k-space (M[, nc])
* ``backward(kdata)``       type-1 NUFFT of dcf-weighted data, i.e. (1/M) A^H D y
* ``forward_backward(im)``  type-21 (normal operator) with dcf in 3-D, none in 2-D,
                            as the reference's nufft3d21 / nufft2d21 drivers
All use eps = 1e-5 as the reference operators do; the 3-D operator clamps nspread
to [3, 6].  numpy in -> numpy out (complex128, like the reference); torch CUDA in ->
torch CUDA out (complex64, no copies).

``joint2operators(espirit(S), NUFFT)`` routes to SENSE-fused kernels: the coil
expansion S*x is fused into the oversampling pad and the coil combination
sum conj(S) * (.) into the crop, so the per-coil images never reach HBM.
"""
import numpy as np
import torch

from .plan import NufftPlan

__all__ = ["NUFFT2d", "NUFFT3d", "NUFFT3d_cuda", "espirit", "joint2operators", "None_opt", "dim_match"]


def dim_match(A_shape, B_shape):
    """Pad the shorter shape with trailing ones (utilities_func.py:393-405)."""
    A_out, B_out = tuple(A_shape), tuple(B_shape)
    if len(A_out) < len(B_out):
        A_out = A_out + (1,) * (len(B_out) - len(A_out))
    elif len(A_out) > len(B_out):
        B_out = B_out + (1,) * (len(A_out) - len(B_out))
    return A_out, B_out


def _to_cuda_c64(a):
    if isinstance(a, torch.Tensor):
        return a.to("cuda", torch.complex64), False
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).astype(np.complex64))).to("cuda"), True


def _to_np(t):
    return t.cpu().numpy().astype(np.complex128)


class _NUFFTnd:
    dim = 3
    eps = 1e-5
    max_nspread = None

    def __init__(self, im_shape=None, dcf=None, ktrajx=None, ktrajy=None, ktrajz=None, axes=None, tuning=None):
        self.axes = axes if axes is not None else tuple(range(self.dim))
        self.im_shape = None if im_shape is None else tuple(int(v) for v in im_shape)
        self.tuning = tuning
        self._k = [None, None, None]
        for i, k in enumerate((ktrajx, ktrajy, ktrajz)[: self.dim]):
            if k is not None:
                self._k[i] = k
        self.dcf = None if dcf is None else (dcf.reshape(-1) if isinstance(dcf, torch.Tensor)
                                             else np.asarray(dcf).reshape(-1))
        self._plans = {}
        self._dcf_dev = None

    # trajectory --------------------------------------------------------------------
    @property
    def ktrajx(self):
        return self._k[0]

    @property
    def ktrajy(self):
        return self._k[1]

    @property
    def ktrajz(self):
        return self._k[2]

    def _flat(self, k):
        return k.reshape(-1) if isinstance(k, torch.Tensor) else np.asarray(k).reshape(-1)

    def normalize_set_ktraj(self, ktraj):
        """ktraj (dim, ...) in any unit; maps max(ktraj) to pi (operators_class.py:323-328)."""
        if isinstance(ktraj, torch.Tensor):
            ktraj = np.pi * ktraj / ktraj.reshape(-1).max()
        else:
            ktraj = np.pi * ktraj / ktraj.flatten().max()
        self._k = [self._flat(ktraj[i]) for i in range(self.dim)] + [None] * (3 - self.dim)
        self._invalidate()
        return tuple(self._k[: self.dim])

    def set_ktraj(self, ktrajx, ktrajy, ktrajz=None, dcf=None):
        ks = (ktrajx, ktrajy, ktrajz)[: self.dim]
        self._k = [self._flat(k) for k in ks] + [None] * (3 - self.dim)
        if dcf is not None:
            self.dcf = self._flat(dcf)
        self._invalidate()

    def pipe_menon_dcf(self, n_iter=20):
        """Estimate a density compensation for the current trajectory (Pipe-Menon iteration
        on this operator's Gaussian kernel, mean 1), make it this operator's dcf and return
        it as a (M,) float32 CUDA tensor.  The reference reads dcf from files; this is for
        trajectories that come without one."""
        d = self.plan(1).pipe_menon_dcf(n_iter)
        self.dcf = d
        self._dcf_dev = None
        return d

    def _invalidate(self):
        for p in self._plans.values():
            p.close()
        self._plans = {}
        self._dcf_dev = None

    def density_weighting(self, kdata, dcf):
        if isinstance(kdata, torch.Tensor):
            w = dcf if isinstance(dcf, torch.Tensor) else torch.as_tensor(np.asarray(dcf))
            w = w.to(kdata.device)
            ks, ws = dim_match(tuple(kdata.shape), tuple(w.shape))
            return (kdata.reshape(ks) * w.reshape(ws)).squeeze()
        ks, ws = dim_match(kdata.shape, dcf.shape)
        return np.multiply(kdata.reshape(ks), dcf.reshape(ws)).squeeze()

    # plans -------------------------------------------------------------------------
    def _coords(self):
        out = []
        for k in self._k[: self.dim]:
            if k is None:
                raise ValueError("trajectory not set")
            if isinstance(k, torch.Tensor):
                t = k.to("cuda")
                t = t if t.dtype in (torch.float32, torch.float64) else t.to(torch.float64)
            else:
                t = torch.from_numpy(np.ascontiguousarray(np.asarray(k, dtype=np.float64))).to("cuda")
            out.append(t.reshape(-1))
        return out

    def plan(self, n_coil):
        p = self._plans.get(n_coil)
        if p is None:
            # tiles tuned for several coils per block do not fit plans with fewer coils (the
            # one-coil density estimation): those take the library's defaults
            tuning = self.tuning
            if tuning is not None and n_coil < getattr(tuning, "coil_group", 0):
                tuning = None
            p = NufftPlan(self.dim, self.im_shape, n_coil=n_coil, n_traj=1, eps=self.eps, iflag=1, df=1.0,
                          max_nspread=self.max_nspread, tuning=tuning)
            p.set_points(self._coords())
            self._plans[n_coil] = p
        return p

    def dcf_device(self):
        if self.dcf is None:
            return None
        if self._dcf_dev is None:
            d = self.dcf
            t = d.to("cuda", torch.float32) if isinstance(d, torch.Tensor) else torch.from_numpy(
                np.ascontiguousarray(np.asarray(d, dtype=np.float32))).to("cuda")
            self._dcf_dev = t.reshape(-1).contiguous()
        return self._dcf_dev

    def _split_image(self, im):
        t, was_np = _to_cuda_c64(im)
        trail = tuple(t.shape[self.dim:])
        nc = int(np.prod(trail)) if trail else 1
        return t.reshape((1,) + self.im_shape + (nc,)), trail, nc, was_np

    # operator ----------------------------------------------------------------------
    def forward(self, im):
        t, trail, nc, was_np = self._split_image(im)
        p = self.plan(nc)
        out = p.type2(t).reshape((p.n_samples,) + trail)
        return _to_np(out) if was_np else out

    def backward(self, kdata):
        was_np = not isinstance(kdata, torch.Tensor)
        t, _ = _to_cuda_c64(kdata)
        M = t.shape[0]
        trail = tuple(t.shape[1:])
        nc = int(np.prod(trail)) if trail else 1
        p = self.plan(nc)
        out = p.type1(t.reshape(M, nc)) if self.dcf is None else self._type1_dcf(p, t.reshape(M, nc))
        # the reference's density_weighting squeezes singleton coil axes (operators_class.py:343)
        shape = tuple(s for s in trail if s != 1) if self.dcf is not None else trail
        out = out.reshape(self.im_shape + shape)
        return _to_np(out) if was_np else out

    def _type1_dcf(self, p, c):
        # density_weighting fused into the spread kernel (per-sample weight)
        return p.type1(c, weight=self.dcf_device())

    def normal_solver(self, n_coil):
        """(plan, None, dcf) of forward_backward on images with n_coil trailing channels,
        for the native solvers."""
        return self.plan(n_coil), None, (self.dcf_device() if self.dim == 3 else None)

    def forward_backward(self, im):
        t, trail, nc, was_np = self._split_image(im)
        p = self.plan(nc)
        out = p.type21(t, dcf=self.dcf_device() if self.dim == 3 else None)
        out = out.reshape(self.im_shape + trail)
        return _to_np(out) if was_np else out


class NUFFT3d(_NUFFTnd):
    """3-D NUFFT operator (pics/operators_class.py:302-364)."""
    dim = 3
    max_nspread = 6


class NUFFT3d_cuda(NUFFT3d):
    """Same operator under the name of pics/operators_cuda_class.py:64-127 (dcf positional)."""

    def __init__(self, im_shape, dcf, ktrajx=None, ktrajy=None, ktrajz=None, axes=(0, 1, 2), tuning=None):
        super().__init__(im_shape, dcf, ktrajx, ktrajy, ktrajz, axes, tuning)


class NUFFT2d(_NUFFTnd):
    """2-D NUFFT operator with the NUFFT3d interface (the reference has no 2-D class);
    forward_backward follows nufft2d21_gaussker, which applies no dcf."""
    dim = 2

    def __init__(self, im_shape=None, dcf=None, ktrajx=None, ktrajy=None, axes=(0, 1), tuning=None):
        super().__init__(im_shape, dcf, ktrajx, ktrajy, None, axes, tuning)

    def set_ktraj(self, ktrajx, ktrajy, dcf=None):
        super().set_ktraj(ktrajx, ktrajy, None, dcf)


class espirit:
    """Coil sensitivity operator (pics/operators_class.py:437-472): forward = S * x,
    backward = sum_c conj(S_c) * x_c (keepdims); the last axis of S is the coil axis."""

    def __init__(self, sensitivity=None, coil_axis=None):
        self.sens = sensitivity
        if coil_axis is None and sensitivity is not None:
            self.coil_axis = len(sensitivity.shape) - 1
        else:
            self.coil_axis = coil_axis
        self._dev = None

    def sens_device(self):
        if self._dev is None:
            t, _ = _to_cuda_c64(self.sens)
            self._dev = t.contiguous()
        return self._dev

    def backward(self, im_coils):
        if isinstance(im_coils, torch.Tensor):
            s = self.sens_device()
            ss, ims = dim_match(tuple(s.shape), tuple(im_coils.shape))
            return (im_coils.reshape(ims) * s.conj().reshape(ss)).sum(dim=self.coil_axis, keepdim=True)
        ss, ims = dim_match(self.sens.shape, im_coils.shape)
        return np.sum(np.multiply(im_coils.reshape(ims), np.conj(self.sens).reshape(ss)), axis=self.coil_axis,
                      keepdims=True)

    def forward(self, im_sos):
        if isinstance(im_sos, torch.Tensor):
            s = self.sens_device()
            ss, ims = dim_match(tuple(s.shape), tuple(im_sos.shape))
            return im_sos.reshape(ims) * s.reshape(ss)
        ss, ims = dim_match(self.sens.shape, im_sos.shape)
        return np.multiply(im_sos.reshape(ims), self.sens.reshape(ss))


class None_opt:
    def forward(self, xin):
        return xin

    def backward(self, xin):
        return xin


class joint2operators:
    """B(A(x)) (pics/operators_class.py:496-514).  With A = espirit and B a NUFFT
    operator the three methods run the SENSE-fused GPU kernels."""

    def __init__(self, Aopt, Bopt):
        self.Aopt = Aopt
        self.Bopt = Bopt
        self._graphs = {}

    def _fused(self):
        return isinstance(self.Aopt, espirit) and isinstance(self.Bopt, _NUFFTnd)

    def _sense_plan(self):
        s = self.Aopt.sens_device()
        nc = s.shape[-1]
        return self.Bopt.plan(nc), s

    def _x(self, x):
        t, was_np = _to_cuda_c64(x)
        shp = self.Bopt.im_shape
        return t.reshape((1,) + shp), was_np

    def forward(self, xin):
        if not self._fused():
            return self.Bopt.forward(self.Aopt.forward(xin))
        p, s = self._sense_plan()
        x, was_np = self._x(xin)
        out = p.sense_forward(x, s)
        return _to_np(out) if was_np else out

    def backward(self, xin):
        if not self._fused():
            return self.Aopt.backward(self.Bopt.backward(xin))
        p, s = self._sense_plan()
        k, was_np = _to_cuda_c64(xin)
        k = k.reshape(p.n_samples, p.n_coil)
        out = p.sense_adjoint(k, s, dcf=self.Bopt.dcf_device()).reshape(self.Bopt.im_shape + (1,))
        return _to_np(out) if was_np else out

    def forward_backward(self, xin):
        if not self._fused():
            if hasattr(self.Bopt, "forward_backward"):
                return self.Aopt.backward(self.Bopt.forward_backward(self.Aopt.forward(xin)))
            return self.Aopt.backward(self.Bopt.backward(self.Bopt.forward(self.Aopt.forward(xin))))
        p, s = self._sense_plan()
        x, was_np = self._x(xin)
        dcf = self.Bopt.dcf_device() if self.Bopt.dim == 3 else None
        out = p.sense_normal(x, s, dcf=dcf).reshape(self.Bopt.im_shape + (1,))
        return _to_np(out) if was_np else out

    def normal_solver(self):
        """(plan, coil maps, dcf) of the fused normal operator for the native solvers, or
        None when the pair is not espirit + NUFFT."""
        if not self._fused():
            return None
        p, s = self._sense_plan()
        return p, s, (self.Bopt.dcf_device() if self.Bopt.dim == 3 else None)

    def normal_graph(self, x_buf, out_buf):
        """CUDA graph of forward_backward on fixed (1, *im_shape) complex64 buffers."""
        if not self._fused():
            raise TypeError("graph capture needs joint2operators(espirit, NUFFT)")
        p, s = self._sense_plan()
        dcf = self.Bopt.dcf_device() if self.Bopt.dim == 3 else None
        return p.capture_normal(x_buf, out_buf, sens=s, dcf=dcf)
