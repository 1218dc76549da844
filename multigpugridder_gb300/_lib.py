"""ctypes binding of libgg_gridder.so (the C ABI declared in include/gg_gridder.h).

The library is built in tree by multigpugridder_gb300/build.py.  There is no
fallback: if the library is missing the import of a function raises.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgg_gridder.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "gg_gridder.h")

GG_OK = 0
GG_ERR_INVALID_ARG = 1
GG_ERR_CUDA = 2
GG_ERR_OUT_OF_MEMORY = 3
GG_ERR_STATE = 4
GG_ERR_NO_DEVICE = 5
GG_ERR_CUFFT = 6
GG_ERR_TIMEOUT = 7
GG_ERR_BUSY = 8

GG_OP_FORWARD = 0
GG_OP_BACK = 1

GG_PREC_F32 = 0
GG_PREC_F16 = 1
GG_PREC_BF16 = 2
PRECISIONS = {"f32": GG_PREC_F32, "fp32": GG_PREC_F32, "f16": GG_PREC_F16, "fp16": GG_PREC_F16,
              "bf16": GG_PREC_BF16}

GG_BP_REF = 0
GG_BP_ADJOINT = 1
BP_MODES = {"ref": GG_BP_REF, "adjoint": GG_BP_ADJOINT}

_c_int = ctypes.c_int
_c_float = ctypes.c_float
_vp = ctypes.c_void_p
_fp = ctypes.c_void_p  # float* passed as integer addresses
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)

# name -> (restype, argtypes)
SIGNATURES = {
    "gg_version": (_c_int, []),
    "gg_global_error": (ctypes.c_char_p, []),
    "gg_create": (_c_int, [_c_int, _c_int, _c_float, _c_int, _c_int, _ip, _c_int, _c_int, ctypes.POINTER(_vp)]),
    "gg_destroy": (None, [_vp]),
    "gg_last_error": (ctypes.c_char_p, [_vp]),
    "gg_get_sizes": (_c_int, [_vp, _ip, _ip, _ip, _ip]),
    "gg_set_kb_table": (_c_int, [_vp, _fp, _c_int]),
    "gg_set_mask_radius": (_c_int, [_vp, _c_float]),
    "gg_set_max_axes_to_allocate": (_c_int, [_vp, _c_int]),
    "gg_set_num_streams_fp": (_c_int, [_vp, _c_int]),
    "gg_set_num_streams_bp": (_c_int, [_vp, _c_int]),
    "gg_set_precision": (_c_int, [_vp, _c_int]),
    "gg_set_image_precision": (_c_int, [_vp, _c_int]),
    "gg_set_bp_mode": (_c_int, [_vp, _c_int]),
    "gg_set_volume": (_c_int, [_vp, _fp, _ip]),
    "gg_set_cas_volume": (_c_int, [_vp, _fp, _ip]),
    "gg_get_cas_volume": (_c_int, [_vp, _fp]),
    "gg_reset_volume": (_c_int, [_vp]),
    "gg_forward_project": (_c_int, [_vp, _fp, _c_int, _fp, _fp]),
    "gg_back_project": (_c_int, [_vp, _fp, _c_int, _fp, _fp, _c_int]),
    "gg_get_volume": (_c_int, [_vp, _fp]),
    "gg_reconstruct_volume": (_c_int, [_vp, _fp, _c_int, _fp, _fp]),
    "gg_set_volume_dev": (_c_int, [_vp, _fp, _vp]),
    "gg_set_cas_volume_dev": (_c_int, [_vp, _fp, _vp]),
    "gg_get_cas_volume_dev": (_c_int, [_vp, _fp, _vp]),
    "gg_forward_project_dev": (_c_int, [_vp, _fp, _c_int, _fp, _fp, _vp]),
    "gg_back_project_dev": (_c_int, [_vp, _fp, _c_int, _fp, _fp, _c_int, _vp]),
    "gg_get_volume_dev": (_c_int, [_vp, _fp, _vp]),
    "gg_reconstruct_volume_dev": (_c_int, [_vp, _fp, _c_int, _fp, _fp, _vp]),
    "gg_back_project_sums_dev": (_c_int, [_vp, _fp, _c_int, _fp, _fp, _vp]),
    "gg_measure_l2_read_gbs": (_c_int, [_c_int, _dp]),
    "gg_volume_from_sums_dev": (_c_int, [_vp, _fp, _fp, _vp]),
    "gg_reconstruct_volume_ctf": (_c_int, [_vp, _fp, _c_int, _fp, _fp, _fp, _fp, _c_float, _c_float, _c_float,
                                           _c_float, _fp]),
    "gg_reconstruct_volume_ctf_dev": (_c_int, [_vp, _fp, _c_int, _fp, _fp, _fp, _fp, _c_float, _c_float, _c_float,
                                               _c_float, _fp, _vp]),
    "gg_forward_project_adjoint": (_c_int, [_vp, _fp, _c_int, _fp, _fp]),
    "gg_forward_project_adjoint_dev": (_c_int, [_vp, _fp, _c_int, _fp, _fp, _vp]),
    "gg_forward_project_kernel": (_c_int, [_fp, _fp, _fp, _fp, _c_float, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _vp]),
    "gg_back_project_kernel": (_c_int, [_fp, _fp, _fp, _fp, _c_float, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _vp]),
    "gg_back_project_adjoint_kernel": (_c_int, [_fp, _fp, _fp, _fp, _c_float, _c_int, _c_int, _c_int, _c_int, _c_int, _vp]),
    "gg_back_project_normalized_noalloc": (_c_int, [_fp, _fp, _fp, _fp, _c_float, _c_int, _c_int, _c_int, _c_int, _c_int,
                                                    _vp]),
    "gg_filter_complex_to_cas": (_c_int, [_fp, _fp, _c_int, _c_int, _vp]),
    "gg_filter_cas_to_complex": (_c_int, [_fp, _fp, _c_int, _c_int, _vp]),
    "gg_filter_fftshift_2d": (_c_int, [_fp, _c_int, _c_int, _c_int, _vp]),
    "gg_filter_fftshift_3d": (_c_int, [_fp, _c_int, _c_int, _vp]),
    "gg_filter_pad_volume": (_c_int, [_fp, _fp, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _vp]),
    "gg_filter_crop_volume": (_c_int, [_fp, _fp, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _vp]),
    "gg_filter_divide_volumes": (_c_int, [_fp, _fp, _c_int, _c_int, _vp]),
    "gg_filter_multiply_volumes": (_c_int, [_fp, _fp, _c_int, _c_int, _c_int, _vp]),
    "gg_filter_add_volumes": (_c_int, [_fp, _fp, _c_int, _c_int, _vp]),
    "gg_filter_divide_scalar": (_c_int, [_fp, _c_float, _c_int, _c_int, _vp]),
    "gg_filter_real_to_complex": (_c_int, [_fp, _fp, _c_int, _c_int, _vp]),
    "gg_filter_complex_to_real": (_c_int, [_fp, _fp, _c_int, _c_int, _vp]),
    "gg_filter_apply_ctf": (_c_int, [_fp, _c_int, _c_int, _fp, _fp, _fp, _c_float, _c_float, _c_float, _c_float, _c_int,
                                     _c_int, _vp]),
    "gg_kb_table": (_c_int, [_c_int, _c_int, _dp]),
    "gg_precomp": (_c_int, [_c_int, _c_int, _dp]),
    "gg_kernel_launch_count": (ctypes.c_longlong, []),
    "gg_server_create": (_c_int, [_c_int, ctypes.c_double, _c_int, ctypes.POINTER(_vp)]),
    "gg_server_destroy": (None, [_vp]),
    "gg_server_last_error": (ctypes.c_char_p, [_vp]),
    "gg_server_add_volume": (_c_int, [_vp, _fp, _c_int, _c_float, _c_int, _ip]),
    "gg_server_remove_volume": (_c_int, [_vp, _c_int]),
    "gg_server_volume_sizes": (_c_int, [_vp, _c_int, _ip, _ip, _ip]),
    "gg_server_submit": (_c_int, [_vp, _c_int, _c_int, _fp, _c_int, _fp, _fp, ctypes.POINTER(ctypes.c_longlong)]),
    "gg_server_wait": (_c_int, [_vp, ctypes.c_longlong, ctypes.c_double, _dp]),
    "gg_server_stats": (_c_int, [_vp, ctypes.POINTER(ctypes.c_longlong), _dp, _dp, _dp, ctypes.POINTER(ctypes.c_longlong),
                                 _dp]),
    "gg_server_reset_stats": (_c_int, [_vp]),
    "gg_server_set_quantum": (_c_int, [_vp, ctypes.c_double]),
    "gg_server_set_max_backlog": (_c_int, [_vp, ctypes.c_double]),
    "gg_server_load": (_c_int, [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), _dp,
                                ctypes.POINTER(ctypes.c_longlong)]),
    "gg_profile_enable": (_c_int, [_vp, _c_int]),
    "gg_profile_read": (_c_int, [_vp, _c_int, _dp, ctypes.POINTER(ctypes.c_longlong)]),
}

GG_KERNEL_FORWARD = 0
GG_KERNEL_BACK = 1
GG_KERNEL_DENSITY = 2

_LIB = None


class GridderError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gg error %d: %s" % (code, msg))
        self.code = code


def declared_symbols():
    """Function names declared in include/gg_gridder.h."""
    with open(HEADER) as f:
        txt = f.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gg_[a-z0-9_]+)\s*\(", txt)))


def lib():
    """Load the in-tree library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libgg_gridder.so is not built (run `python -c \"import __graft_entry__ as g; g.build()\"` "
                              "or `python multigpugridder_gb300/build.py`)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(rc, handle=None):
    if rc != GG_OK:
        L = lib()
        msg = L.gg_last_error(handle) if handle else L.gg_global_error()
        raise GridderError(rc, (msg or b"").decode(errors="replace"))
    return rc
