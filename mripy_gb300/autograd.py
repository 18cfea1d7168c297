"""Differentiable NUFFT: ``torch.autograd.Function`` wrappers over a ``NufftPlan``.

``nufft_forward(image, coords, plan)`` computes the type-2 transform c = A(x) F and is
differentiable with respect to both inputs:

* image:  grad_F = A^H grad_c, computed by the hand-written adjoint pipeline
  (spread -> FFT -> crop; the plan's type-1 carries mripy's 1/M, undone per group);
* coords: grad_x[j, d] = Re( sum_coil conj(grad_c[j]) dc_j/dx_{j,d} ) from the
  trajectory-gradient kernel, which differentiates the Gaussian weights analytically
  (d/dx exp(-u^2/(4 tau)) = -u/(2 tau) exp(-u^2/(4 tau))) over the same oversampled
  grid the forward pass interpolates.

PyTorch's convention for a real input of a complex function is grad_x = Re(conj(g) dc/dx)
and for a complex-linear map grad_F = A^H g; both are what the kernels return.

``nufft_adjoint(samples, coords, plan)`` is the type-1 transform (with 1/M), differentiable
with respect to the samples (grad_c = (1/M) A grad_F).

Shapes: image (n_traj, *shape, n_coil) complex64; coords (dim, M_total) real, radians;
samples (M_total, n_coil) complex64.  The plan's trajectory groups are kept.
"""
import torch

from . import _native as N


def _set_points(plan, coords):
    cs = [coords[d].detach().contiguous() for d in range(plan.dim)]
    plan.set_points(cs, traj_offsets=plan.traj_offsets if plan.traj_offsets is not None and
                    plan.traj_offsets[-1] == cs[0].numel() else None)


def _points_for_backward(ctx, coords):
    """The backward pass reuses the forward pass's bin sort when nothing re-sorted the plan
    in between (the plan's points generation is unchanged); otherwise it sorts again."""
    if ctx.plan.points_generation != ctx.points_generation:
        _set_points(ctx.plan, coords)


def _group_scale(plan, img, inverse):
    """Multiply each trajectory group's image by M_g (inverse=True) to undo type-1's 1/M_g.
    The per-group factors depend on the group sizes alone: they are built once per set of
    group offsets, not per set of points (a host-to-device copy each step would cost more
    than the multiply)."""
    off = tuple(int(v) for v in plan.traj_offsets)
    cache = getattr(plan, "_group_scale_cache", None)
    if cache is None or cache[0] != off or cache[1] != img.device:
        counts = torch.tensor([off[g + 1] - off[g] for g in range(plan.n_traj)], dtype=torch.float32,
                              device=img.device)
        inv = torch.where(counts > 0, 1.0 / counts.clamp(min=1.0), torch.zeros_like(counts))
        cache = (off, img.device, counts, inv)
        plan._group_scale_cache = cache
    s = cache[2] if inverse else cache[3]
    return img * s.view((-1,) + (1,) * (img.dim() - 1))


class _Type2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, image, coords, plan):
        _set_points(plan, coords)
        img = image.detach().contiguous()
        out = plan.type2(img)
        ctx.plan = plan
        ctx.points_generation = plan.points_generation
        ctx.save_for_backward(img, coords)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        img, coords = ctx.saved_tensors
        plan = ctx.plan
        _points_for_backward(ctx, coords)
        g = grad_out.contiguous().to(torch.complex64)
        grad_img = grad_coords = None
        if ctx.needs_input_grad[0]:
            grad_img = _group_scale(plan, plan.type1(g), inverse=True)
        if ctx.needs_input_grad[1]:
            grid = plan.pad_deapod(img)
            plan.fft(grid, N.GBN_FFT_INVERSE if plan.iflag < 0 else N.GBN_FFT_FORWARD)
            gx = plan.interp_grad_coords(grid, g)                   # (M, dim) float32
            grad_coords = gx.t().to(coords.dtype)
        return grad_img, grad_coords, None


class _Type1(torch.autograd.Function):
    @staticmethod
    def forward(ctx, samples, coords, plan):
        _set_points(plan, coords)
        out = plan.type1(samples.detach().contiguous())
        ctx.plan = plan
        ctx.points_generation = plan.points_generation
        ctx.save_for_backward(coords)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (coords,) = ctx.saved_tensors
        plan = ctx.plan
        _points_for_backward(ctx, coords)
        grad_c = None
        if ctx.needs_input_grad[0]:
            g = _group_scale(plan, grad_out.contiguous().to(torch.complex64), inverse=False)
            grad_c = plan.type2(g.contiguous())
        if ctx.needs_input_grad[1]:
            raise NotImplementedError("coordinate gradients of the adjoint transform are not provided; "
                                      "differentiate nufft_forward instead")
        return grad_c, None, None


def nufft_forward(image, coords, plan):
    """Differentiable type-2 NUFFT (see module docstring)."""
    return _Type2.apply(image, coords, plan)


def nufft_adjoint(samples, coords, plan):
    """Type-1 NUFFT with mripy's 1/M, differentiable with respect to the samples."""
    return _Type1.apply(samples, coords, plan)


class NufftOp(torch.nn.Module):
    """Module form: ``NufftOp(plan)(image, coords)`` -> samples."""

    def __init__(self, plan):
        super().__init__()
        self.plan = plan

    def forward(self, image, coords):
        return nufft_forward(image, coords, self.plan)
