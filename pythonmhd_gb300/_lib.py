"""ctypes binding of ``libpythonmhd_gb300.so`` (declared in ``include/pythonmhd_gb300.h``).

The library is built in-tree (``pythonmhd_gb300/build.py``).  Loading never
falls back to anything else: if the library is missing or cannot be loaded,
``load()`` raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

c_double_p = ctypes.POINTER(ctypes.c_double)

# name -> (restype, argtypes)
SIGNATURES = {
    "mhd2d_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_void_p)]),
    "mhd2d_upload": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p, c_double_p, c_double_p]),
    "mhd1d_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "mhd1d_upload": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p]),
    "mhd3d_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_void_p)]),
    "mhd3d_upload": (ctypes.c_int, [ctypes.c_void_p] + [c_double_p] * 5),
    "mhd3d_upload_device": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_void_p] * 5),
    "mhd3d_advance": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_longlong,
                                     ctypes.c_longlong, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double)]),
    "mhd3d_download": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int] + [c_double_p] * 5),
    "mhd3d_state_ptrs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int] + [ctypes.POINTER(ctypes.c_void_p)] * 5),
    "mhd3d_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_size_t),
                                  ctypes.POINTER(ctypes.c_void_p)]),
    "mhd3d_destroy": (None, [ctypes.c_void_p]),
    "mhd2d_upload_device": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_void_p] * 4),
    "mhd2d_advance": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_longlong,
                                     ctypes.c_longlong, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double)]),
    "mhd2d_download": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                                      c_double_p]),
    "mhd2d_cfl_dt": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "mhd2d_advance_dt": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_longlong,
                                        ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "mhd2d_download_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4),
    "mhd2d_set_dt_log": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]),
    "mhd2d_state_ptrs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int] + [ctypes.POINTER(ctypes.c_void_p)] * 4),
    "mhd2d_peek": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p, ctypes.c_size_t]),
    "mhd2d_last_launches": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "mhd2d_device_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "mhd2d_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "mhd2d_cfl_dt_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mhdb_create": (ctypes.c_int, [ctypes.c_int] + [ctypes.c_void_p] * 7 + [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "mhdb_upload": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p, c_double_p, c_double_p, c_double_p]),
    "mhdb_advance": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_void_p] * 4 + [ctypes.c_double, ctypes.c_void_p,
                                    ctypes.c_void_p]),
    "mhdb_download": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                                     c_double_p]),
    "mhdb_configure": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "mhdb_upload_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4),
    "mhdb_pack_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "mhdb_state_ptrs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
                        + [ctypes.POINTER(ctypes.c_void_p)] * 4),
    "mhdb_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_size_t),
                                 ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_void_p)]),
    "mhdb_instance_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "mhdb_get_tiles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong,
                                      ctypes.POINTER(ctypes.c_longlong)]),
    "mhdb_set_tiles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong]),
    "mhdb_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mhd2d_check_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                        ctypes.POINTER(ctypes.c_longlong)]),
    "mhd2d_validate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "mhd2d_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int)]),
    "mhdb_destroy": (None, [ctypes.c_void_p]),
    "mhd2d_adj_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "mhd2d_adj_cycle": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    "mhd2d_adj_cycle_reverse": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p]),
    "mhd2d_adj_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                         c_double_p, ctypes.c_int, ctypes.c_void_p, c_double_p]),
    "mhd2d_adj_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mhd2d_adj_configure": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t]),
    "mhd2d_adj_reshape": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    "mhd2d_adj_cycle_bytes": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_size_t)]),
    "mhd2d_adj_restore": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, c_double_p]),
    "mhd2d_adj_set_tail": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "mhd2d_adj_branches": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, c_double_p,
                                          ctypes.c_void_p]),
    "mhd2d_adj_record": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 3),
    "mhd2d_adj_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t),
                                      ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_int)]),
    "mhd2d_adj_destroy": (None, [ctypes.c_void_p]),
    "mhd2d_adj_quotient": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]),
    "mhd_quotient6": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]),
    "mhd_softfp": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]),
    "mhd3d_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_longlong, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.POINTER(ctypes.c_longlong)]),
    "mhd2d_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_longlong, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.POINTER(ctypes.c_longlong)]),
    "mhd_ic_work_words": (ctypes.c_longlong, []),
    "mhd_ic_scatter_spectrum": (ctypes.c_int, [ctypes.c_longlong] + [ctypes.c_void_p] * 5),
    "mhd_ic_turbulence_2d": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]
                             + [ctypes.c_void_p] * 9 + [ctypes.c_longlong, ctypes.c_void_p]),
    "mhd_ic_orszag_tang": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double] + [ctypes.c_void_p] * 6),
    "mhd2d_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "mhd2d_destroy": (None, [ctypes.c_void_p]),
}


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first when stale and nvcc is present) and return the CDLL."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing and _build.is_stale():
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"pythonmhd_gb300: CUDA library not built ({path}); run pythonmhd_gb300/build.py")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class MhdError(RuntimeError):
    def __init__(self, status: int, where: str):
        lib = load(build_if_missing=False)
        msg = lib.mhd2d_strerror(status).decode()
        super().__init__(f"{where}: {msg} (status {status})")
        self.status = status


def check(status: int, where: str):
    if status != 0:
        raise MhdError(status, where)
