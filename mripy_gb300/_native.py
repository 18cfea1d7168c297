"""ctypes binding of ``libgbnufft.so`` (the C ABI declared in ``include/gbnufft.h``).

The library is the only compute path: if it cannot be loaded, every transform
raises.  There is no CPU or PyTorch fallback.
"""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgbnufft.so")

GBN_OK = 0
GBN_COORD_F32 = 0
GBN_COORD_F64 = 1
GBN_FFT_FORWARD = -1
GBN_FFT_INVERSE = 1
GBN_BAND_INPUT = 1    # gbn_fft_band: the grid is zero outside the image band (after the pad)
GBN_BAND_OUTPUT = 2   # gbn_fft_band: only the image band of the result is read (by the crop)

# every function the header declares, for the export check in the CPU tests
EXPORTED = (
    "gbn_version", "gbn_status_string", "gbn_last_error", "gbn_grid_params",
    "gbn_plan_create", "gbn_plan_destroy", "gbn_plan_get_info", "gbn_plan_status", "gbn_plan_check_wait_expiry",
    "gbn_set_points", "gbn_plan_grid",
    "gbn_spread", "gbn_interp", "gbn_fft", "gbn_fft_band", "gbn_pad_deapod", "gbn_crop_deapod",
    "gbn_type1", "gbn_type2", "gbn_type21",
    "gbn_sense_forward", "gbn_sense_adjoint", "gbn_sense_normal",
    "gbn_interp_grad_coords",
    "gbn_graph_capture_normal", "gbn_graph_launch", "gbn_graph_destroy",
    "gbn_cg_sense", "gbn_ista_haar", "gbn_dcf_pipe_menon", "gbn_espirit_eigen", "gbn_haar_dwt", "gbn_prox_haar",
    "gbn_spread2d_noalloc",
    "gbn_type1_host", "gbn_type2_host", "gbn_type21_host",
    "gbn_nufft2d1_gaussker", "gbn_nufft2d2_gaussker", "gbn_nufft2d21_gaussker",
    "gbn_nufft3d1_gaussker", "gbn_nufft3d2_gaussker", "gbn_nufft3d21_gaussker",
)


class PlanDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32), ("ms", ctypes.c_int32), ("mt", ctypes.c_int32), ("mu", ctypes.c_int32),
        ("eps", ctypes.c_double), ("max_nspread", ctypes.c_int32), ("iflag", ctypes.c_int32),
        ("df", ctypes.c_double), ("n_coil", ctypes.c_int32), ("n_traj", ctypes.c_int32),
        ("spread_tile", ctypes.c_int32 * 3), ("interp_tile", ctypes.c_int32 * 3),
        ("max_subproblem", ctypes.c_int32), ("coil_group", ctypes.c_int32), ("threads", ctypes.c_int32),
        ("interp_threads", ctypes.c_int32), ("interp_coil_group", ctypes.c_int32),
        ("interp_staging", ctypes.c_int32), ("dense_tile_samples", ctypes.c_int32),
        ("spread_variant", ctypes.c_int32), ("interp_variant", ctypes.c_int32),
        ("fft_variant", ctypes.c_int32),
    ]


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("nspread", ctypes.c_int32), ("nf", ctypes.c_int32 * 3), ("tau", ctypes.c_double),
        ("n_samples", ctypes.c_int64), ("grid_cells", ctypes.c_int64), ("n_inst", ctypes.c_int64),
        ("spread_subproblems", ctypes.c_int64), ("interp_subproblems", ctypes.c_int64),
        ("spread_entries", ctypes.c_int64), ("spread_tile", ctypes.c_int32 * 3),
        ("interp_tile", ctypes.c_int32 * 3), ("coil_group", ctypes.c_int32), ("threads", ctypes.c_int32),
        ("interp_threads", ctypes.c_int32), ("max_subproblem", ctypes.c_int32), ("device_bytes", ctypes.c_int64),
        ("interp_coil_group", ctypes.c_int32), ("dense_subproblems", ctypes.c_int64),
        ("spread_kernels", ctypes.c_int32), ("split_tiles", ctypes.c_int64), ("spread_variant", ctypes.c_int32),
        ("interp_variant", ctypes.c_int32), ("fft_variant", ctypes.c_int32),
    ]


class Layout(ctypes.Structure):
    _fields_ = [("traj_stride", ctypes.c_int64), ("coil_stride", ctypes.c_int64),
                ("elem_stride", ctypes.c_int64)]


class GbnError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("gbnufft status %d: %s" % (status, message))
        self.status = status


_lib = None
_lock = threading.Lock()

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f64 = ctypes.c_double
_f32 = ctypes.c_float

GBN_SOLVE_X0 = 1
GBN_SOLVE_NO_GRAPH = 2
GBN_SOLVE_FISTA = 4


def _declare(lib):
    P = ctypes.POINTER
    sig = {
        "gbn_version": ([], _i32),
        "gbn_status_string": ([_i32], ctypes.c_char_p),
        "gbn_last_error": ([ctypes.c_char_p, _i32], _i32),
        "gbn_grid_params": ([_i32, _i32, _i32, _i32, _f64, _i32, P(_i32), P(_i64), P(_f64)], _i32),
        "gbn_plan_create": ([P(PlanDesc), P(_vp)], _i32),
        "gbn_plan_destroy": ([_vp], _i32),
        "gbn_plan_get_info": ([_vp, P(PlanInfo)], _i32),
        "gbn_plan_status": ([_vp, _vp], _i32),
        "gbn_plan_check_wait_expiry": ([_vp, ctypes.c_uint32, _vp], _i32),
        "gbn_set_points": ([_vp, _i32, _vp, _vp, _vp, P(_i64), _vp], _i32),
        "gbn_plan_grid": ([_vp], _vp),
        "gbn_spread": ([_vp, _vp, Layout, _vp, _vp], _i32),
        "gbn_interp": ([_vp, _vp, _vp, Layout, _vp, _vp], _i32),
        "gbn_fft": ([_vp, _vp, _i32, _vp], _i32),
        "gbn_fft_band": ([_vp, _vp, _i32, _i32, _vp], _i32),
        "gbn_pad_deapod": ([_vp, _vp, Layout, _vp, _vp], _i32),
        "gbn_crop_deapod": ([_vp, _vp, _vp, Layout, _vp], _i32),
        "gbn_type1": ([_vp, _vp, Layout, _vp, _vp, Layout, _vp], _i32),
        "gbn_type2": ([_vp, _vp, Layout, _vp, Layout, _vp], _i32),
        "gbn_type21": ([_vp, _vp, Layout, _vp, Layout, _vp, _vp], _i32),
        "gbn_sense_forward": ([_vp, _vp, Layout, _vp, Layout, _vp, Layout, _vp], _i32),
        "gbn_sense_adjoint": ([_vp, _vp, Layout, _vp, _vp, Layout, _vp, Layout, _vp], _i32),
        "gbn_sense_normal": ([_vp, _vp, Layout, _vp, Layout, _vp, _vp, Layout, _vp], _i32),
        "gbn_interp_grad_coords": ([_vp, _vp, _vp, Layout, _vp, _vp], _i32),
        "gbn_graph_capture_normal": ([_vp, _vp, Layout, _vp, Layout, _vp, _vp, Layout, P(_vp)], _i32),
        "gbn_graph_launch": ([_vp, _vp], _i32),
        "gbn_graph_destroy": ([_vp], _i32),
        "gbn_cg_sense": ([_vp, _vp, Layout, _vp, _vp, _vp, _i32, _vp, _i32, _vp], _i32),
        "gbn_ista_haar": ([_vp, _vp, Layout, _vp, _vp, _vp, _i32, _f32, _f32, _i32, _i32, _vp], _i32),
        "gbn_dcf_pipe_menon": ([_vp, _i32, _vp, _vp], _i32),
        "gbn_espirit_eigen": ([_vp, _i64, _i32, _i32, _i32, _vp, _vp, _vp], _i32),
        "gbn_haar_dwt": ([_i32, P(_i32), _i32, _i64, _i64, _vp, _vp, _i32, _vp], _i32),
        "gbn_prox_haar": ([_i32, P(_i32), _i32, _i64, _i64, _vp, _f32, _vp, _vp], _i32),
        "gbn_spread2d_noalloc": ([_i32, _vp, _vp, _i64, _vp, Layout, _i32, _i32, _i32, _f64, _f64, _vp, _vp], _i32),
        "gbn_type1_host": ([_vp, _vp, _vp, _vp], _i32),
        "gbn_type2_host": ([_vp, _vp, _vp, _vp], _i32),
        "gbn_type21_host": ([_vp, _vp, _vp, _vp, _vp], _i32),
        "gbn_nufft2d1_gaussker": ([_vp, _vp, _vp, _i64, _i32, _i32, _i32, _f64, _f64, _i32, _vp], _i32),
        "gbn_nufft2d2_gaussker": ([_vp, _vp, _vp, _i64, _i32, _i32, _i32, _f64, _f64, _i32, _vp], _i32),
        "gbn_nufft2d21_gaussker": ([_vp, _vp, _vp, _i64, _i32, _i32, _i32, _f64, _f64, _i32, _vp], _i32),
        "gbn_nufft3d1_gaussker": ([_vp, _vp, _vp, _vp, _i64, _i32, _i32, _i32, _i32, _f64, _f64, _i32, _vp], _i32),
        "gbn_nufft3d2_gaussker": ([_vp, _vp, _vp, _vp, _i64, _i32, _i32, _i32, _i32, _f64, _f64, _i32, _vp], _i32),
        "gbn_nufft3d21_gaussker": ([_vp, _vp, _vp, _vp, _i64, _i32, _i32, _i32, _i32, _vp, _f64, _f64, _i32,
                                    _vp], _i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


def lib():
    """Load (building first if needed, in a source checkout) and return the library."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                from . import build as _build
                _build.build()
            l = ctypes.CDLL(LIB_PATH)
            _declare(l)
            _lib = l
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().gbn_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status):
    if status != GBN_OK:
        raise GbnError(status, last_error() or lib().gbn_status_string(status).decode())
    return status
