"""ctypes binding of libgopf_gpu.so (the C ABI in include/gopf_gpu.h)."""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgopf_gpu.so")

GOPF_OK = 0
STATUS = {
    0: "GOPF_OK",
    1: "GOPF_ERR_ARG",
    2: "GOPF_ERR_CUDA",
    3: "GOPF_ERR_OOM",
    4: "GOPF_ERR_NAN",
    5: "GOPF_ERR_TIMEOUT",
    6: "GOPF_ERR_UNSUPPORTED",
    7: "GOPF_ERR_STATE",
    8: "GOPF_ERR_PARSE",
}
GOPF_FP32, GOPF_FP64 = 0, 1
GOPF_STEPPER_EULER, GOPF_STEPPER_RK4, GOPF_STEPPER_IMPLICIT_EULER, GOPF_STEPPER_SDD = 0, 1, 2, 3
DER_PRODUCT, DER_POLY, DER_INDICATOR, DER_INDICATOR_D, DER_INDICATOR_HD, DER_WHITE_NOISE, DER_MPOLY = range(7)
NOISE_WHITE, NOISE_CONSERVATIVE = 1, 2
SRC_NONE, SRC_FIELD, SRC_DERIVED = range(3)
RED_SUM, RED_SUMSQ, RED_MIN, RED_MAX, RED_NONFINITE = range(5)
OPT_CHECK_FINITE, OPT_USE_GRAPHS, OPT_FAST_KERNELS, OPT_TMA, OPT_DIRECT_HOST = 0, 1, 2, 3, 5
OPT_WAIT_LIMIT_NS = 6
OPT_X_ROWS = 7
OPT_PDL = 9
OPT_Z_LINES = 8
MAX_FACTORS = 8
BATCH_AUTO, BATCH_LINE, BATCH_STOCKHAM_CT, BATCH_STOCKHAM = -1, 0, 1, 2
BATCH_MODE_AUTO, BATCH_MODE_CHAINS, BATCH_MODE_PERSISTENT = -1, 0, 1


class GopfDerived(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("nfac", ctypes.c_int),
        ("field", ctypes.c_int * MAX_FACTORS),
        ("power", ctypes.c_int * MAX_FACTORS),
        ("coef", ctypes.c_double * MAX_FACTORS),
    ]


class GopfTerm(ctypes.Structure):
    _fields_ = [
        ("eq", ctypes.c_int),
        ("implicit", ctypes.c_int),
        ("coef", ctypes.c_double),
        ("lap", ctypes.c_int),
        ("source", ctypes.c_int),
        ("src_index", ctypes.c_int),
    ]


# every exported symbol with its (argtypes, restype)
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_cp = ctypes.c_char_p
_i = ctypes.c_int
_ll = ctypes.c_longlong
_sz = ctypes.c_size_t
SIGNATURES = {
    "gopf_ctx_create": ([_i, _ip, _i, _i, ctypes.POINTER(_vp)], _i),
    "gopf_ctx_destroy": ([_vp], _i),
    "gopf_last_error": ([_vp], _cp),
    "gopf_status_string": ([_i], _cp),
    "gopf_set_stream": ([_vp, _vp], _i),
    "gopf_set_option": ([_vp, _i, _ll], _i),
    "gopf_add_field": ([_vp, _cp, _ip], _i),
    "gopf_add_scalar": ([_vp, _cp, ctypes.c_double, ctypes.c_double], _i),
    "gopf_register_function": ([_vp, _cp, _i, _cp, _dp, _ip, _i], _i),
    "gopf_register_polynomial": ([_vp, _cp, _dp, _ip, _i, _i], _i),
    "gopf_register_elastic": ([_vp, _cp, _cp, _dp, _dp], _i),
    "gopf_register_volcons": ([_vp, _cp, _cp, _cp, ctypes.c_double], _i),
    "gopf_volcons_multiplier": ([_vp, _dp], _i),
    "gopf_add_equation": ([_vp, _cp], _i),
    "gopf_register_noise": ([_vp, _cp, _i, _cp, ctypes.c_double, ctypes.c_ulonglong], _i),
    "gopf_init": ([_vp], _i),
    "gopf_equation_summary": ([_vp, _i, _ip, _ip], _i),
    "gopf_get_terms": ([_vp, ctypes.POINTER(GopfTerm), _i, _ip], _i),
    "gopf_get_derived": ([_vp, ctypes.POINTER(GopfDerived), _i, _ip], _i),
    "gopf_set_terms": ([_vp, _i, ctypes.POINTER(GopfDerived), _i, ctypes.POINTER(GopfTerm), _i], _i),
    "gopf_set_stepper": ([_vp, _i, ctypes.c_double], _i),
    "gopf_field_upload": ([_vp, _i, _dp, _sz], _i),
    "gopf_field_download": ([_vp, _i, _dp, _sz], _i),
    "gopf_field_upload_real": ([_vp, _i, _dp, _sz], _i),
    "gopf_field_download_real": ([_vp, _i, _dp, _sz], _i),
    "gopf_step": ([_vp, _ll], _i),
    "gopf_prepare_graphs": ([_vp, _ll], _i),
    "gopf_get_time": ([_vp, _dp], _i),
    "gopf_get_step": ([_vp, ctypes.POINTER(_ll)], _i),
    "gopf_synchronize": ([_vp], _i),
    "gopf_reduce": ([_vp, _i, _i, _dp], _i),
    "gopf_point_values": ([_vp, _i, ctypes.POINTER(_ll), _i, _dp], _i),
    "gopf_free_energy": ([_vp, _i, _dp, _i, ctypes.c_double, _dp], _i),
    "gopf_elastic_energy": ([_vp, _i, _i, _dp, _dp, _dp], _i),
    "gopf_add_source": ([_vp, _i, _dp, _i, _ip], _i),
    "gopf_set_source_amplitudes": ([_vp, _dp, _i, _i], _i),
    "gopf_sdd_init": ([_vp, _dp, _dp, _sz], _i),
    "gopf_sdd_set_orientation": ([_vp, _dp, _sz], _i),
    "gopf_sdd_set_params": ([_vp] + [ctypes.c_double] * 5, _i),
    "gopf_sdd_get_orientation": ([_vp, _dp, _sz], _i),
    "gopf_sdd_monitor": ([_vp, _dp], _i),
    "gopf_sdd_dimer_length": ([_vp, ctypes.c_double, _dp], _i),
    "gopf_fft": ([_vp, _i, _dp, _sz], _i),
    "gopf_freq": ([_vp, _ll, _dp], _i),
    "gopf_conjugate_node": ([_vp, _ll], _ll),
    "gopf_device_bytes": ([_vp, ctypes.POINTER(_sz)], _i),
    "gopf_kernels_per_step": ([_vp, _ip], _i),
    "gopf_profile_step": ([_vp, _i, _dp, _dp, _i, _ip], _i),
    "gopf_profile_slot_name": ([_vp, _i, ctypes.c_char_p, _i], _i),
    "gopf_adjoint_forward": ([_vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, _i, _i, _dp, _dp], _i),
    "gopf_adjoint_backward": ([_vp, _dp, _dp, _dp, _dp], _i),
    "gopf_adjoint_release": ([_vp], _i),
    "gopf_reduce_noalloc": ([_vp, _sz, _dp, _vp], _i),
    "gopf_noalloc_last_error": ([], _cp),
    "gopf_register_hessian": ([_vp, _cp, _dp, _i], _i),
    "gopf_register_spectral_viscosity": ([_vp, _cp, ctypes.c_double, ctypes.c_double, _i], _i),
    "gopf_save_float64": ([_vp, _i, _cp, _i], _i),
    "gopf_io_wait": ([_vp], _i),
    "gopf_load_float64": ([_vp, _i, _cp], _i),
    "gopf_set_modal_filter": ([_vp, _dp, _i], _i),
    "gopf_vandeven_table": ([_i, _dp, _i], _i),
    "gopf_kernel_launches": ([_vp, _ll, ctypes.POINTER(ctypes.c_longlong)], _i),
    "gopf_set_newton_krylov": ([_vp, _i, ctypes.c_double, ctypes.c_double, _i, _i], _i),
    "gopf_newton_stats": ([_vp, _ip, _ip, _dp, _ip], _i),
    "gopf_batch_create": ([ctypes.POINTER(_vp), _i, ctypes.POINTER(_vp)], _i),
    "gopf_batch_destroy": ([_vp], _i),
    "gopf_batch_last_error": ([_vp], _cp),
    "gopf_batch_set_stream": ([_vp, _vp], _i),
    "gopf_batch_step": ([_vp, _ll], _i),
    "gopf_batch_kernels_per_step": ([_vp, _ip], _i),
    "gopf_batch_tune": ([_vp, _i], _i),
    "gopf_batch_tune_reset": ([], _i),
    "gopf_batch_force": ([_vp, _i, _i, _i, _i, _i, _i], _i),
    "gopf_batch_choice": ([_vp, _i, _ip], _i),
    "gopf_batch_set_mode": ([_vp, _i], _i),
    "gopf_batch_mode": ([_vp, _ip], _i),
    "gopf_batch_set_wait_limit": ([_vp, ctypes.c_longlong], _i),
    "gopf_sweep_partition": ([ctypes.POINTER(_ll), _i, _i, _ip, ctypes.POINTER(_ll)], _i),
}

_lib = None


def load(path: str | None = None):
    """Load the in-tree library (fails loudly when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(p)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L
