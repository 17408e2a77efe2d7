"""Loader of the in-tree C-ABI library ``librimp2_gpu_gb300.so``.

The library is the only compute path: if it is missing this module raises
instead of falling back to anything on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librimp2_gpu_gb300.so")

_lock = threading.Lock()
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_llp = C.POINTER(C.c_longlong)
_vp = C.c_void_p

# name -> (argtypes, restype); mirrors include/rimp2_gpu.h
SIGNATURES = {
    "rimp2_last_error_string": ([], C.c_char_p),
    "rimp2_version": ([], C.c_char_p),
    "rimp2_set_stream": ([_vp], C.c_int),
    "rimp2_get_dev_mem": ([C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)], C.c_int),
    "rimp2_kernel_launch_count": ([], C.c_longlong),
    "rimp2_sync_status": ([_vp], C.c_int),
    "rimp2_set_timing": ([C.c_int], C.c_int),
    "rimp2_selftest_bounded_wait": ([C.c_longlong, _vp], C.c_int),
    "rimp2_selftest_rcp_denom": ([C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                  C.POINTER(C.c_float)], C.c_int),
    "rimp2_last_timing": ([C.POINTER(C.c_float)], C.c_int),
    "rimp2_last_split_kernel": ([], C.c_int),
    "rimp2_probe_fp64_peak": ([_dp], C.c_int),
    "rimp2_calc_tocca": ([_ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp], C.c_int),
    "rimp2_calc_tvirta": ([_ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp], C.c_int),
    "rimp2_calc_toccb": ([_ip, _ip, _dp, _dp, _dp], C.c_int),
    "rimp2_calc_tvirtb": ([_ip, _ip, _dp, _dp, _dp], C.c_int),
    "rimp2_transalpha1": ([_ip, _ip, _ip, _dp, _dp, _dp], C.c_int),
    "rimp2_transalpha2": ([_ip, _ip, _ip, _ip, _dp, _dp, _dp], C.c_int),
    "rimp2_calc_gocc": ([_ip, _ip, _ip, _dp, _dp], C.c_int),
    "rimp2_calc_gvirt": ([_ip, _ip, _ip, _dp, _dp], C.c_int),
    "rimp2_calc_gen4dimfo": ([_ip, _dp, _ip, _ip, _dp, _ip, _ip, _dp], C.c_int),
    "rimp2_dgemm": ([C.c_char_p, C.c_char_p, _ip, _ip, _ip, _dp, _dp, _ip, _dp, _ip, _dp, _dp,
                     _ip], C.c_int),
    "rimp2_steps5to8": ([_ip] * 5 + [_dp] * 11, C.c_int),
    "rimp2_first_order": ([_ip] * 6 + [_dp] * 10, C.c_int),
    "rimp2_energy_eos": ([_ip] * 5 + [_dp] * 9 + [_ip], C.c_int),
    "rimp2_datafile_header": ([C.c_char_p, _ip], C.c_int),
    "rimp2_datafile_read": ([C.c_char_p, C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "rimp2_datafile_write": ([C.c_char_p, _ip, C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "rimp2_energy": ([_ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _ip], C.c_int),
    "rimp2_energy_dev": ([C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int, _vp],
                         C.c_int),
    "rimp2_energy_split_dev": ([C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, C.c_int, _vp],
                               C.c_int),
    "rimp2_energy_fp64_noalloc_dev": ([C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp],
                                      C.c_int),
    "rimp2_split_nslices": ([C.c_int, C.c_int, C.c_int], C.c_int),
    "rimp2_energy_batched": ([_ip, _ip, _ip, _ip, _dp, _llp, _dp, _llp, _dp, _llp, _dp, _llp, _dp,
                              _ip], C.c_int),
    "rimp2_gen_fragment_dev": ([C.c_ulonglong, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp],
                               C.c_int),
    "rimp2_batch_plan_create": ([C.POINTER(_vp), C.c_int, _ip, _ip, _ip, C.POINTER(_vp),
                                 C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp),
                                 _ip, C.c_int, _vp], C.c_int),
    "rimp2_batch_plan_execute": ([_vp, _vp], C.c_int),
    "rimp2_batch_plan_destroy": ([_vp], C.c_int),
    "rimp2_set_split_buckets": ([C.c_int, _ip, _ip], C.c_int),
    "rimp2_set_split_kernel_rule": ([C.c_int, _ip, _ip, _ip], C.c_int),
    "rimp2_split_kernel_for": ([C.c_int, C.c_int, C.c_int], C.c_int),
    "rimp2_calpha_from_ao": ([_ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp], C.c_int),
    "rimp2_calpha_from_ao_dev": ([C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp],
                                 C.c_int),
    "rimp2_calpha_from_ao_split_dev": ([C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp,
                                        _vp], C.c_int),
    "rimp2_ao2mo_dev": ([C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, _vp],
                        C.c_int),
    "rimp2_cholesky_dev": ([C.c_int, _vp, _vp], C.c_int),
    "rimp2_trsm_lower_dev": ([C.c_int, C.c_int, _vp, _vp, _vp, _vp], C.c_int),
    "rimp2_gen_ao_dev": ([C.c_ulonglong, C.c_int, C.c_int, _vp, _vp, _vp], C.c_int),
}


class Rimp2Error(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, name, status, msg):
        super().__init__(f"{name} failed with status {status}: {msg}")
        self.status = status


def lib():
    """Load (once) and return the ctypes handle; raise if the library is absent."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g;"
                    f" g.build()'` (there is no CPU fallback)")
            L = C.CDLL(LIB_PATH)
            for name, (args, res) in SIGNATURES.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = res
            _lib = L
    return _lib


def check(name, status):
    if status != 0:
        msg = lib().rimp2_last_error_string().decode(errors="replace")
        raise Rimp2Error(name, status, msg)
    return status


def call(name, *args):
    return check(name, getattr(lib(), name)(*args))
