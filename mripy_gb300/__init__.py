"""mripy_gb300: GB300-native Gaussian-gridding NUFFT, a drop-in for mripy's NUFFT path.

Layers (bottom up):
  csrc/ + include/gbnufft.h   sm_103a CUDA kernels behind a C ABI (libgbnufft.so)
  _native                     ctypes binding; the library is the only compute path
  plan.NufftPlan              plans over PyTorch CUDA tensors
  nufft_func                  nufft{1,2,3}d{1,2,21}_gaussker[_cuda] (fft/nufft_func(_cuda).py)
  operators                   NUFFT2d / NUFFT3d / NUFFT3d_cuda, espirit, joint2operators
  autograd                    torch.autograd.Function with image and trajectory gradients
  solvers                     CG-SENSE, IST/FISTA with a Haar wavelet, graph-captured normal op
  tune                        autotuner for tile sizes per trajectory density
"""
from .plan import NufftPlan, Tuning, grid_params  # noqa: F401
from . import nufft_func, operators  # noqa: F401

__version__ = "0.1.0"
