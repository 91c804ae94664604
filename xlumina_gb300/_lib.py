"""ctypes binding of libxlgb.so (declarations mirror ``include/xlgb.h``).

The library is the only compute path: if it is missing or fails to load,
every propagator raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

from ._build import LIB

XL_OK = 0
XL_EINVAL = -1
XL_ENOMEM = -2
XL_ETIMEOUT = -3
XL_ECUDA = -4
XL_EUNSUPPORTED = -5
XL_MAX_OPS = 8
XL_MAX_SIDE = 4096
XL_RS_NOALLOC_MAX_WORK_BYTES = 64 << 20

XL_PASS_RS_COLS, XL_PASS_CZT_ROWS, XL_PASS_CZT_COLS, XL_PASS_RS_ROWS = range(4)

OP_NONE, OP_PHASE, OP_SSLM, OP_SSLM_AMP, OP_LCD, OP_LP, OP_SEPMASK, OP_CMUL, OP_HIGHNA, OP_HIGHNA_EZ = range(10)


class XlOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("pmask", ctypes.c_int), ("ptr", ctypes.c_void_p * 4),
                ("sval", ctypes.c_float * 4), ("pbstride", ctypes.c_longlong), ("dval", ctypes.c_double * 4)]


class XlProg(ctypes.Structure):
    _fields_ = [("nops", ctypes.c_int), ("ops", XlOp * XL_MAX_OPS)]


class XlRsArgs(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_int), ("comps_in", ctypes.c_int), ("comps_out", ctypes.c_int),
                ("ny", ctypes.c_int), ("nx", ctypes.c_int),
                ("inp", ctypes.c_void_p * 3), ("in_bstride", ctypes.c_longlong),
                ("out", ctypes.c_void_p * 3), ("out_bstride", ctypes.c_longlong),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
                ("spectrum", ctypes.c_void_p), ("spectrum_stride", ctypes.c_longlong),
                ("spectrum_index", ctypes.c_void_p), ("work", ctypes.c_void_p),
                ("pre", XlProg), ("post", XlProg), ("adjoint", ctypes.c_int), ("spectra", ctypes.c_void_p)]


XL_CZT_SCALAR, XL_CZT_VECTOR, XL_CZT_PLAIN = 0, 1, 2


class XlCztArgs(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_int), ("comps_in", ctypes.c_int), ("comps_out", ctypes.c_int),
                ("mode", ctypes.c_int), ("ny", ctypes.c_int), ("nx", ctypes.c_int), ("my", ctypes.c_int),
                ("mx", ctypes.c_int), ("log2_lx", ctypes.c_int), ("log2_ly", ctypes.c_int),
                ("inp", ctypes.c_void_p * 3), ("in_bstride", ctypes.c_longlong),
                ("out", ctypes.c_void_p * 3), ("out_bstride", ctypes.c_longlong),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("xout", ctypes.c_void_p),
                ("yout", ctypes.c_void_p), ("z", ctypes.c_double), ("wavelength", ctypes.c_double),
                ("cte_re", ctypes.c_double), ("cte_im", ctypes.c_double),
                ("pre_x", ctypes.c_void_p), ("g_x", ctypes.c_void_p), ("post_x", ctypes.c_void_p),
                ("pre_y", ctypes.c_void_p), ("g_y", ctypes.c_void_p), ("post_y", ctypes.c_void_p),
                ("work", ctypes.c_void_p), ("pre", XlProg), ("adjoint", ctypes.c_int),
                ("z_batch", ctypes.c_void_p), ("cte_batch", ctypes.c_void_p),
                ("f_in", ctypes.c_void_p), ("f_out", ctypes.c_void_p)]


class XlCztChirpArgs(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_int), ("ny", ctypes.c_int), ("nx", ctypes.c_int), ("my", ctypes.c_int),
                ("mx", ctypes.c_int), ("log2_lx", ctypes.c_int), ("log2_ly", ctypes.c_int),
                ("adjoint", ctypes.c_int), ("z", ctypes.c_void_p), ("wavelength", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("xout0", ctypes.c_double),
                ("xout1", ctypes.c_double), ("yout0", ctypes.c_double), ("yout1", ctypes.c_double),
                ("pre_x", ctypes.c_void_p), ("g_x", ctypes.c_void_p), ("post_x", ctypes.c_void_p),
                ("pre_y", ctypes.c_void_p), ("g_y", ctypes.c_void_p), ("post_y", ctypes.c_void_p),
                ("cte", ctypes.c_void_p)]


class XlBsArgs(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_int), ("ny", ctypes.c_int), ("nx", ctypes.c_int),
                ("inp", (ctypes.c_void_p * 2) * 2), ("in_bstride", ctypes.c_longlong * 2),
                ("out", (ctypes.c_void_p * 2) * 2), ("out_bstride", ctypes.c_longlong),
                ("m", ctypes.c_void_p), ("m_bstride", ctypes.c_longlong), ("theta", ctypes.c_void_p),
                ("theta_bstride", ctypes.c_longlong), ("kind", ctypes.c_int)]


XL_BS_MATRIX, XL_BS_SYMMETRIC, XL_BS_SINGLE_PORT0, XL_BS_SINGLE_PORT1 = 0, 1, 2, 3


XL_NOISE_MAX_TABLES = 256


class XlNoiseArgs(ctypes.Structure):
    _fields_ = [("tables", ctypes.c_int), ("resolution", ctypes.c_int), ("planes", ctypes.c_int),
                ("n_distances", ctypes.c_int), ("n_wps", ctypes.c_int), ("min_d", ctypes.c_double),
                ("max_d", ctypes.c_double), ("min_phase", ctypes.c_double), ("max_phase", ctypes.c_double),
                ("discretize", ctypes.c_int), ("distances", ctypes.c_void_p), ("slms", ctypes.c_void_p),
                ("amps", ctypes.c_void_p), ("wps", ctypes.c_void_p)]


XL_ADAMW_MAX_TENSORS = 32


class XlAdamWTensor(ctypes.Structure):
    _fields_ = [("p", ctypes.c_void_p), ("g", ctypes.c_void_p), ("m", ctypes.c_void_p), ("v", ctypes.c_void_p),
                ("n", ctypes.c_longlong)]


class XlAdamWArgs(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int), ("t", XlAdamWTensor * XL_ADAMW_MAX_TENSORS), ("lr", ctypes.c_float),
                ("beta1", ctypes.c_float), ("beta2", ctypes.c_float), ("eps", ctypes.c_float),
                ("weight_decay", ctypes.c_float), ("step", ctypes.c_void_p)]


# name -> (restype, argtypes); every symbol include/xlgb.h declares.
SIGNATURES = {
    "xl_last_error": (ctypes.c_char_p, []),
    "xl_version": (ctypes.c_int, []),
    "xl_struct_size": (ctypes.c_size_t, [ctypes.c_char_p]),
    "xl_init": (ctypes.c_int, []),
    "xl_kernel_variant_count": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "xl_set_kernel_variant": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "xl_get_kernel_variant": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "xl_device_timeouts": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint), ctypes.c_int]),
    "xl_device_status": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint), ctypes.c_int]),
    "xl_set_wait_limit": (ctypes.c_int, [ctypes.c_ulonglong]),
    "xl_host_mapped": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "xl_rs_spectrum_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    "xl_rs_spectrum_work_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    "xl_rs_transfer_spectrum": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    "xl_rs_transfer_spectrum_dz": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    "xl_rs_transfer_spectra_device_z": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                       ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                       ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong,
                                                       ctypes.c_void_p]),
    "xl_re_inner": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p,
                                   ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                                   ctypes.c_void_p]),
    "xl_vrs_dz_ez": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p]),
    "xl_rs_z_gradient": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                        ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p]),
    "xl_rs_work_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "xl_rs_propagate": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlRsArgs)]),
    "xl_rs_stage": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlRsArgs), ctypes.c_int]),
    "xl_rs_propagate_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlRsArgs)]),
    "xl_fft_lines": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p]),
    "xl_czt_work_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "xl_czt": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlCztArgs)]),
    "xl_czt_stage": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlCztArgs), ctypes.c_int]),
    "xl_czt_chirps": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlCztChirpArgs)]),
    "xl_czt_transfer_plane": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
    "xl_ops_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_longlong,
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_longlong,
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_longlong,
                                       ctypes.POINTER(XlProg), ctypes.POINTER(ctypes.c_void_p)]),
    "xl_highna_coefficients": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
    "xl_mse_intensity_work_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_longlong]),
    "xl_mse_intensity": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p,
                                        ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    "xl_mse_intensity_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p,
                                             ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "xl_plane_mse": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p,
                                    ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                                    ctypes.c_void_p]),
    "xl_plane_mse_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_longlong,
                                         ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "xl_loss_work_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_longlong]),
    "xl_area_loss": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p]),
    "xl_area_loss_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p]),
    "xl_norm_intensity_mse": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_int,
                                             ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong,
                                             ctypes.c_void_p, ctypes.c_void_p]),
    "xl_norm_intensity_mse_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_int,
                                                  ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                                                  ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p]),
    "xl_beam_splitter": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlBsArgs)]),
    "xl_beam_splitter_work_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "xl_beam_splitter_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlBsArgs),
                                                 ctypes.POINTER(ctypes.c_void_p), ctypes.c_longlong,
                                                 ctypes.POINTER(ctypes.c_void_p), ctypes.c_longlong,
                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "xl_table_noise": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlNoiseArgs), ctypes.POINTER(ctypes.c_uint32)]),
    "xl_philox4x32_10": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                        ctypes.POINTER(ctypes.c_uint32)]),
    "xl_adamw_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(XlAdamWArgs)]),
    "xl_apply_ops": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_void_p), ctypes.c_longlong,
                                    ctypes.POINTER(ctypes.c_void_p), ctypes.c_longlong,
                                    ctypes.POINTER(XlProg)]),
}

_lib = None


class XlError(RuntimeError):
    """A libxlgb entry point returned an error code (``code``: the XL_E* value)."""

    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code


def load(path: str = LIB):
    """Load libxlgb.so and declare its entry points (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"libxlgb.so not found at {path}: build it with `python -m xlumina_gb300._build` "
            "(nvcc, sm_103a); there is no fallback compute path")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str = "") -> None:
    if rc != XL_OK:
        msg = _lib.xl_last_error().decode() if _lib is not None else ""
        raise XlError(f"{what or 'libxlgb'} failed with code {rc}: {msg}", rc)


def check_device_status(clear: bool = True) -> None:
    """Raise XlError (code XL_ETIMEOUT) if a kernel had a bounded wait run out
    since the last check: that launch returned without its data and its output
    is not valid.  Reads a word the kernels write in mapped host memory, so it
    costs no device synchronisation; launches still queued are covered by a
    later check.  ``clear``: reset the word when raising."""
    if _lib is None:
        return
    flag = ctypes.c_uint(0)
    check(_lib.xl_device_status(ctypes.byref(flag), 0), "xl_device_status")
    if flag.value:
        if clear:
            _lib.xl_device_status(ctypes.byref(flag), 1)
        raise XlError("a libxlgb kernel's bounded wait on its input copies ran out (about one second); "
                      "the output of that launch is not valid", XL_ETIMEOUT)
