"""ctypes binding of libwstack_gb300.so (the C ABI in include/wstack_gb300.h and
include/wstack_gb300_io.h).

The library is required: there is no CPU or pure-PyTorch fallback.  If it is
missing, loading raises immediately with the command that builds it.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwstack_gb300.so")

WSG_OK = 0
WSG_ERR_ARG = 1
WSG_ERR_CUDA = 2
WSG_ERR_CUFFT = 3
WSG_ERR_NOMEM = 4
WSG_ERR_STATE = 5
WSG_ERR_CAPACITY = 6
WSG_ERR_UNSUPPORTED = 7
WSG_ERR_IO = 8

WSG_FP64 = 0
WSG_FP32C = 1

STATUS_NAMES = {0: "WSG_OK", 1: "WSG_ERR_ARG", 2: "WSG_ERR_CUDA", 3: "WSG_ERR_CUFFT",
                4: "WSG_ERR_NOMEM", 5: "WSG_ERR_STATE", 6: "WSG_ERR_CAPACITY",
                7: "WSG_ERR_UNSUPPORTED", 8: "WSG_ERR_IO"}


class WstackError(RuntimeError):
    """A call into libwstack_gb300.so returned a non-zero wsg_status."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class Stats(ctypes.Structure):
    _fields_ = [("points_in", ctypes.c_longlong), ("records", ctypes.c_longlong),
                ("dropped_plane", ctypes.c_longlong), ("dropped_window", ctypes.c_longlong),
                ("bins", ctypes.c_int), ("tile", ctypes.c_int), ("max_bin_records", ctypes.c_int),
                ("ctas", ctypes.c_int)]


class Tuning(ctypes.Structure):
    _fields_ = [("tile", ctypes.c_int), ("ctas", ctypes.c_int), ("chunk", ctypes.c_int),
                ("ms", ctypes.c_float)]


class Channel(ctypes.Structure):
    _fields_ = [("num_points", ctypes.c_long), ("uu", ctypes.c_void_p), ("vv", ctypes.c_void_p),
                ("ww", ctypes.c_void_p), ("vis_real", ctypes.c_void_p),
                ("vis_img", ctypes.c_void_p), ("weight", ctypes.c_void_p)]


# include/wstack_gb300_io.h
WSG_MAX_DATASETS = 100
WSG_PATH_LEN = 1024
WSG_NAME_LEN = 256
WSG_DROPPED_ROWS = 1000
WSG_MAX_SECTORS = 1023

PARAM_NAMES = ("ufile", "vfile", "wfile", "weightsfile", "visrealfile", "visimgfile", "metafile",
               "outfile", "outfile1", "outfile2", "outfile3", "fftfile", "fftfile2", "fftfile3",
               "logfile", "extension", "timingfile")


class Params(ctypes.Structure):
    _fields_ = ([(f, ctypes.c_int) for f in ("num_threads", "ndatasets", "grid_size_x",
                                               "grid_size_y", "num_w_planes", "w_support",
                                               "verbose_level", "n_datapaths")]
                + [("datapath", (ctypes.c_char * WSG_PATH_LEN) * WSG_MAX_DATASETS)]
                + [(f, ctypes.c_char * WSG_NAME_LEN) for f in PARAM_NAMES])


class Metadata(ctypes.Structure):
    _fields_ = [("Nmeasures", ctypes.c_long), ("Nvis", ctypes.c_long), ("Nweights", ctypes.c_long),
                ("freq_per_chan", ctypes.c_long), ("polarisations", ctypes.c_long),
                ("Ntimes", ctypes.c_long), ("dt", ctypes.c_double), ("thours", ctypes.c_double),
                ("baselines", ctypes.c_long), ("uvmin", ctypes.c_double),
                ("uvmax", ctypes.c_double), ("wmin", ctypes.c_double), ("wmax", ctypes.c_double)]


class RunOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("write_data", ctypes.c_int),
                ("write_image", ctypes.c_int), ("write_timings", ctypes.c_int),
                ("verbose", ctypes.c_int), ("outdir", ctypes.c_char * WSG_PATH_LEN)]


class RunReport(ctypes.Structure):
    _fields_ = [("datasets", ctypes.c_int), ("Nmeasures", ctypes.c_long), ("Nvis", ctypes.c_long),
                ("resolution", ctypes.c_double), ("dropped", ctypes.c_longlong)] + \
               [(f, ctypes.c_double) for f in ("setup", "compose", "kernel", "reduce", "fft",
                                               "phase", "write", "total")]


_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_L = ctypes.c_long

# name -> (restype, argtypes); every symbol of include/*.h
SIGNATURES = {
    "wstack": (None, [_I, _L, _L, _L, _P, _P, _P, _P, _P, _P, _D, _D, _I, _I, _I, _P, _I]),
    "phase_correction": (None, [_P, _P, _P, _I, _I, _I, _I, _I, _D, _D, _D, _I]),
    "test": (_I, [_I]),
    "wstack_fft_planes": (_I, [_P, _P, _I, _I, _I]),
    "wstack_gb300_last_error": (_I, []),
    "wstack_gb300_last_error_string": (ctypes.c_char_p, []),
    "wstack_gb300_set_precision": (_I, [_I]),
    "wstack_gb300_release": (None, []),
    "wsg_plan_create": (_I, [ctypes.POINTER(_P), _I, _I, _I, _I, _D, _D, _I, _P]),
    "wsg_plan_destroy": (_I, [_P]),
    "wsg_plan_set_stream": (_I, [_P, _P]),
    "wsg_plan_set_tuning": (_I, [_P, _I, _I, _I]),
    "wsg_plan_reserve": (_I, [_P, _L]),
    "wsg_plan_set_wcorrection": (_I, [_P, _D, _D, _D]),
    "wsg_plan_get_stats": (_I, [_P, ctypes.POINTER(Stats)]),
    "wsg_plan_device_bytes": (ctypes.c_longlong, [_P]),
    "wsg_plan_grid": (_P, [_P]),
    "wsg_bin": (_I, [_P, _L, _L, _L, _P, _P, _P, _P, _P, _P]),
    "wsg_grid": (_I, [_P, _P]),
    "wsg_grid_occupied": (_I, [_P, _P]),
    "wsg_plan_set_layout": (_I, [_P, _L]),
    "wsg_fft": (_I, [_P, _P, _I]),
    "wsg_wcorrect": (_I, [_P, _P, _P, _D]),
    "wsg_wcorrect_adjoint": (_I, [_P, _P, _P, _D]),
    "wsg_degrid": (_I, [_P, _P, _P]),
    "wsg_fft_wcorrect": (_I, [_P, _P, _P, _I]),
    "wsg_wcorrect_adjoint_fft": (_I, [_P, _P, _P, _I]),
    "wsg_image_forward": (_I, [_P, _L, _L, _L, _P, _P, _P, _P, _P, _P, _P]),
    "wsg_image_adjoint": (_I, [_P, _P, _P]),
    "wsg_image_forward_host": (_I, [_P, _L, _L, _L, _P, _P, _P, _P, _P, _P, _P]),
    "wsg_image_adjoint_host": (_I, [_P, _P, _P]),
    "wsg_image_forward_host_async": (_I, [_P, _L, _L, _L, _P, _P, _P, _P, _P, _P, _P]),
    "wsg_image_adjoint_host_async": (_I, [_P, _P, _P]),
    "wsg_plan_synchronize": (_I, [_P]),
    "wsg_plan_autotune": (_I, [_P, _L, _L, _L, _P, _P, _P, _P, _P, _P, _P, _I,
                               ctypes.POINTER(Tuning), ctypes.POINTER(Tuning), _I,
                               ctypes.POINTER(_I)]),
    "wsg_batch_create": (_I, [ctypes.POINTER(_P), _I, _I, _I, _I, _D, _D, _I, _I, _P]),
    "wsg_batch_destroy": (_I, [_P]),
    "wsg_batch_set_stream": (_I, [_P, _P]),
    "wsg_batch_set_wcorrection": (_I, [_P, _D, _D, _D]),
    "wsg_batch_set_tuning": (_I, [_P, _I, _I, _I]),
    "wsg_batch_bind": (_I, [_P, ctypes.POINTER(Channel)]),
    "wsg_batch_forward": (_I, [_P, _P, _I]),
    "wsg_batch_adjoint": (_I, [_P, _P, _P]),
    "wsg_batch_autotune": (_I, [_P, _P, _I, ctypes.POINTER(Tuning), ctypes.POINTER(Tuning), _I,
                                ctypes.POINTER(_I)]),
    "wsg_batch_vis_offset": (ctypes.c_longlong, [_P, _I]),
    "wsg_batch_grids": (_P, [_P]),
    "wsg_batch_get_stats": (_I, [_P, ctypes.POINTER(Stats)]),
    "wsg_batch_device_bytes": (ctypes.c_longlong, [_P]),
    "wsg_grid_noalloc": (_I, [_I, _L, _L, _L, _P, _P, _P, _P, _P, _P, _D, _D, _I, _I, _I, _P, _P]),
    "wsg_sector_count": (_I, [_P, _L, _L, _I, _D, _D, _P, _P]),
    "wsg_sector_lists": (_I, [_P, _L, _L, _I, _D, _D, _P, _P, _L, _P]),
    "wsg_sector_gather": (_I, [_P, _L, _L, _I, _D, _L, _L, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                               _P, _P, _P, _P]),
    "wsg_initialize_array": (_I, [_P, _L, _L, _I, _D, _D, _P, ctypes.POINTER(_P)]),
    # include/wstack_gb300_io.h
    "wsg_read_parameter_file": (_I, [ctypes.c_char_p, ctypes.POINTER(Params)]),
    "wsg_read_metadata": (_I, [ctypes.c_char_p, ctypes.POINTER(Metadata)]),
    "wsg_partition_measurements": (_I, [ctypes.POINTER(Metadata), _I, _I, ctypes.POINTER(_L)]),
    "wsg_read_measurements": (_I, [ctypes.POINTER(Params), _I, ctypes.POINTER(Metadata), _L,
                                   _P, _P, _P, _P, _P, _P]),
    "wsg_reference_resolution": (_I, [_D, _D, ctypes.POINTER(_D)]),
    "wsg_write_cube_dump": (_I, [_P, _I, _I, _I, _D, ctypes.c_char_p, ctypes.c_char_p]),
    "wsg_plan_dump_cube": (_I, [_P, _P, _D, ctypes.c_char_p, ctypes.c_char_p]),
    "wsg_write_image_dump": (_I, [_P, _P, _L, ctypes.c_char_p, ctypes.c_char_p]),
    "wsg_write_timings": (_I, [ctypes.c_char_p, ctypes.POINTER(_D)]),
    "wsg_run_options_default": (None, [ctypes.POINTER(RunOptions)]),
    "wsg_run_paramfile": (_I, [ctypes.c_char_p, ctypes.POINTER(RunOptions),
                               ctypes.POINTER(RunReport)]),
}

_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load libwstack_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "or `python lofar_gb300/build.py` (requires nvcc)")
    lib = ctypes.CDLL(p, mode=ctypes.RTLD_GLOBAL)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int) -> None:
    if status != WSG_OK:
        msg = load().wstack_gb300_last_error_string()
        raise WstackError(status, msg.decode() if msg else "")


def last_error() -> tuple[int, str]:
    lib = load()
    msg = lib.wstack_gb300_last_error_string()
    return lib.wstack_gb300_last_error(), (msg.decode() if msg else "")
