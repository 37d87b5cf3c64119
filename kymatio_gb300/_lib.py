"""ctypes binding of the C ABI in ``include/kymatio_gb300.h``.

The shared library is built in-tree (``kymatio_gb300/_lib``) by
``kymatio_gb300.build``.  There is no fallback: every transform in this
package runs through these entry points, and a missing library raises.
"""
import ctypes
import os
import threading

from . import build as _build

KYM_OK = 0
KYM_ERR_INVALID = 1
KYM_ERR_UNSUPPORTED = 2
KYM_ERR_CUDA = 3
KYM_ERR_WORKSPACE = 4

_ERRNAMES = {KYM_ERR_INVALID: 'invalid argument', KYM_ERR_UNSUPPORTED: 'unsupported geometry',
             KYM_ERR_CUDA: 'CUDA error', KYM_ERR_WORKSPACE: 'workspace too small'}

_c_int, _c_size, _vp = ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes); the full list of exported entry points
SIGNATURES = {
    'kym_version': (ctypes.c_char_p, []),
    'kym_last_error': (ctypes.c_char_p, []),
    'kym_set_specialized': (_c_int, [_c_int]),
    'kym_set_tc_dft': (_c_int, [_c_int]),
    'kym_s2d_plan_create': (_c_int, [_c_int] * 6 + [ctypes.POINTER(_vp)]),
    'kym_s2d_plan_destroy': (_c_int, [_vp]),
    'kym_s2d_plan_info': (_c_int, [_vp] + [_ip] * 6),
    'kym_s2d_filter_shape': (_c_int, [_vp, _c_int, _ip, _ip]),
    'kym_s2d_set_chunk': (_c_int, [_vp, _c_int]),
    'kym_s2d_get_chunk': (_c_int, [_vp]),
    'kym_s2d_workspace_bytes': (_c_size, [_vp, _c_int]),
    'kym_s2d_forward': (_c_int, [_vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp, _c_size, _vp]),
    'kym_s2d_forward_noalloc': (_c_int, [_vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp]),
    'kym_s2d_backward_workspace_bytes': (_c_size, [_vp, _c_int]),
    'kym_s2d_set_backward_chunk': (_c_int, [_vp, _c_int]),
    'kym_s2d_backward': (_c_int, [_vp, _vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp, _c_size, _vp]),
    'kym_s2d_saved_bytes': (_c_size, [_vp, _c_int]),
    'kym_s2d_forward_save': (_c_int, [_vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp, _c_size, _vp, _c_size,
                                      _vp]),
    'kym_s2d_backward_saved': (_c_int, [_vp, _vp, _c_size, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp,
                                        _c_size, _vp]),
    'kym_s2d_forward_tc': (_c_int, [_vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, ctypes.POINTER(_vp),
                                    ctypes.POINTER(_vp), _c_int, _vp, _c_size, _vp, _vp,
                                    ctypes.POINTER(ctypes.c_float), _c_int]),
    'kym_s2d_group_kernels': (_c_int, [_vp, _c_int, _c_int]),
    'kym_s2d_group_launches': (_c_int, [_vp, _c_int, _c_int, _c_int]),
    'kym_s2d_filter_bank_floats': (ctypes.c_longlong, [_c_int] * 4),
    'kym_s2d_filter_bank_workspace_bytes': (_c_size, [_c_int] * 4),
    'kym_s2d_filter_bank': (_c_int, [_c_int] * 4 + [_vp, ctypes.c_longlong, _vp, _c_size, _vp]),
    'kym_s2d_group_uses_tc': (_c_int, [_vp, _c_int]),
    'kym_s2d_set_group_tc': (_c_int, [_vp, _c_int, _c_int]),
    'kym_set_side_lane': (_c_int, [_c_int]),
    'kym_s2d_group_lane': (_c_int, [_vp, _c_int]),
    'kym_s2d_forward_host': (_c_int, [_vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, ctypes.POINTER(_vp),
                                      ctypes.POINTER(_vp), _c_int, _vp, _vp, _vp, _vp, _c_size, _c_int, _vp, _vp]),
    'kym_tc_selftest': (_c_int, [_vp, _vp, _vp, _c_int, _c_int, _c_int, _vp, _vp]),
    'kym_s2d_group_count': (_c_int, [_vp]),
    'kym_s2d_group_info': (_c_int, [_vp, _c_int] + [_ip] * 6),
    'kym_s2d_forward_timed': (_c_int, [_vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp, _c_size, _vp,
                                       ctypes.POINTER(ctypes.c_float), _c_int]),
    'kym_s1d_plan_create': (_c_int, [_c_int] * 6 + [_ip, _ip, _c_int, _ip, _ip, _c_int, _c_int, _c_int,
                                                   ctypes.POINTER(_vp)]),
    'kym_s1d_plan_destroy': (_c_int, [_vp]),
    'kym_s1d_plan_info': (_c_int, [_vp, _ip, _ip, _ip]),
    'kym_s1d_set_chunk': (_c_int, [_vp, _c_int]),
    'kym_s1d_workspace_bytes': (_c_size, [_vp, _c_int]),
    'kym_s1d_forward': (_c_int, [_vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp, _c_size, _vp]),
    'kym_s1d_backward_workspace_bytes': (_c_size, [_vp, _c_int]),
    'kym_s1d_backward': (_c_int, [_vp, _vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp, _c_size, _vp]),
    'kym_s1d_saved_bytes': (_c_size, [_vp, _c_int]),
    'kym_s1d_forward_save': (_c_int, [_vp, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp, _c_size, _vp, _c_size,
                                      _vp]),
    'kym_s1d_backward_saved': (_c_int, [_vp, _vp, _c_size, _vp, _vp, _c_int, ctypes.POINTER(_vp), _c_int, _vp,
                                        _c_size, _vp]),
    'kym_op_fft2': (_c_int, [_vp, _vp, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, ctypes.c_float, _vp]),
    'kym_op_cdgmm': (_c_int, [_vp, _vp, _vp, ctypes.c_longlong, ctypes.c_longlong, _c_int, _vp]),
    'kym_op_modulus': (_c_int, [_vp, _vp, ctypes.c_longlong, _vp]),
    'kym_op_modulus_backward': (_c_int, [_vp, _vp, _vp, ctypes.c_longlong, _vp]),
    'kym_op_subsample': (_c_int, [_vp, _vp, _c_int, _c_int, _c_int, _c_int, _c_int, _vp]),
    'kym_op_subsample_adjoint': (_c_int, [_vp, _vp, _c_int, _c_int, _c_int, _c_int, _c_int, _vp]),
    'kym_op_reflect_pad': (_c_int, [_vp, _vp] + [_c_int] * 7 + [_vp]),
    'kym_op_reflect_pad_adjoint': (_c_int, [_vp, _vp] + [_c_int] * 7 + [_vp]),
}

_lock = threading.Lock()
_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load (once) and return the ctypes handle of the library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(
                    'kymatio_gb300 CUDA library not built (%s missing); run '
                    '`python -m kymatio_gb300.build`' % path)
            _build.build()
        h = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
        return h


class KymError(RuntimeError):
    pass


def check(status, what):
    if status != KYM_OK:
        msg = _ERRNAMES.get(status, 'status %d' % status)
        if status == KYM_ERR_CUDA:
            msg += ': ' + load().kym_last_error().decode()
        raise KymError('%s failed: %s' % (what, msg))


def int_array(values):
    arr = (ctypes.c_int * max(1, len(values)))(*values)
    return arr


def ptr_array(ptrs):
    return (_vp * max(1, len(ptrs)))(*ptrs)
