"""Oracle package: test infrastructure (FP64 restatement of mripy's CPU NUFFT).

Used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
as the checker or the timed CPU reference; the product never imports it.
"""
from .nufft_oracle import *  # noqa: F401,F403
from .nufft_oracle import build  # noqa: F401
