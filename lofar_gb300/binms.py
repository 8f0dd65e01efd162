"""The reference's files, through libwstack_gb300.so (include/wstack_gb300_io.h).

A reference run reads a parameter file, then per dataset a ``meta.txt`` and
six raw binary files from a directory (a ``.binMS``), and can dump the grid,
the transformed planes and the image as float64 files.  The functions here
mirror the reference's functions of the same role:

=========================  ============================================
``read_parameter_file``    read_parameter_file()   init.c:124-250
``read_metadata``          readMetaData()          init.c:278-307
``partition_measurements`` metaData_calculation()  init.c:311-343
``read_measurements``      readData()              init.c:387-501
``reference_resolution``   resolution              gridding.c:160
``write_cube_dump``        write_gridded_data() / write_fftw_data()
                                                   gridding.c:366-447,
                                                   fourier_transform.c:74-159
``write_image_dump``       WRITE_IMAGE block       fourier_transform.c:177-219
``write_timings``          write_result()          result.c:49-62
``run``                    main()                  main.c:8-94
=========================  ============================================

``write_dataset`` writes arrays in the reference's input layout (the
reference only reads it; its files come from a measurement-set converter).
Every call goes through the C library; failures raise ``WstackError``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib
from ._lib import WSG_DROPPED_ROWS, WSG_FP32C, WSG_FP64, check

META_FIELDS = ("Nmeasures", "Nvis", "freq_per_chan", "polarisations", "Ntimes", "dt", "thours",
               "baselines", "uvmin", "uvmax", "wmin", "wmax")


def _b(path) -> bytes:
    return os.fsencode(path)


def _params_dict(p: _lib.Params) -> dict:
    d = {f: getattr(p, f) for f in ("num_threads", "ndatasets", "grid_size_x", "grid_size_y",
                                    "num_w_planes", "w_support", "verbose_level")}
    d["datapath"] = [p.datapath[i].value.decode() for i in range(p.n_datapaths)]
    for f in _lib.PARAM_NAMES:
        d[f] = getattr(p, f).decode()
    return d


def _params_struct(d: dict) -> _lib.Params:
    p = _lib.Params()
    for f in ("num_threads", "ndatasets", "grid_size_x", "grid_size_y", "num_w_planes",
              "w_support", "verbose_level"):
        setattr(p, f, int(d.get(f, 0)))
    paths = list(d.get("datapath", []))
    p.n_datapaths = len(paths)
    for i, s in enumerate(paths):
        p.datapath[i].value = os.fsencode(s)
    for f in _lib.PARAM_NAMES:
        setattr(p, f, os.fsencode(d.get(f, "")))
    return p


def read_parameter_file(path) -> dict:
    """Parameter file -> dict (numbers, ``datapath`` list and file names)."""
    p = _lib.Params()
    check(_lib.load().wsg_read_parameter_file(_b(path), ctypes.byref(p)))
    return _params_dict(p)


def _meta_dict(m: _lib.Metadata) -> dict:
    return {f: getattr(m, f) for f, _ in _lib.Metadata._fields_}


def _meta_struct(d: dict) -> _lib.Metadata:
    m = _lib.Metadata()
    for f, t in _lib.Metadata._fields_:
        setattr(m, f, (float if t is ctypes.c_double else int)(d.get(f, 0)))
    return m


def read_metadata(path) -> dict:
    """meta.txt -> dict with the 12 fields (and Nweights = 0)."""
    m = _lib.Metadata()
    check(_lib.load().wsg_read_metadata(_b(path), ctypes.byref(m)))
    return _meta_dict(m)


def partition_measurements(meta: dict, rank: int = 0, size: int = 1) -> tuple[dict, int]:
    """Drop the last 1000 rows and take rank's share -> (meta for the rank, startrow)."""
    m = _meta_struct(meta)
    start = ctypes.c_long(0)
    check(_lib.load().wsg_partition_measurements(ctypes.byref(m), int(rank), int(size),
                                                 ctypes.byref(start)))
    return _meta_dict(m), start.value


def read_measurements(params: dict, dataset: int, meta: dict, startrow: int) -> dict:
    """The rank's rows of the six binary files -> NumPy arrays (uu, vv, ww
    float64; weights, vis_real, vis_img float32 in the reference's flat layout).
    A short file raises; use ``run`` for the reference's zero-fill-and-continue."""
    n, nw, nv = int(meta["Nmeasures"]), int(meta["Nweights"]), int(meta["Nvis"])
    out = {"uu": np.empty(n), "vv": np.empty(n), "ww": np.empty(n),
           "weights": np.empty(nw, np.float32), "vis_real": np.empty(nv, np.float32),
           "vis_img": np.empty(nv, np.float32)}
    p = _params_struct(params)
    m = _meta_struct(meta)
    check(_lib.load().wsg_read_measurements(
        ctypes.byref(p), int(dataset), ctypes.byref(m), int(startrow),
        *[out[k].ctypes.data for k in ("uu", "vv", "ww", "weights", "vis_real", "vis_img")]))
    return out


def reference_resolution(uvmin: float, uvmax: float) -> float:
    r = ctypes.c_double()
    check(_lib.load().wsg_reference_resolution(float(uvmin), float(uvmax), ctypes.byref(r)))
    return r.value


def write_cube_dump(cube: np.ndarray, real_path, img_path, scale: float = 1.0) -> None:
    """[planes][ny][nx] complex128 host cube -> the two float64 dump files."""
    c = np.ascontiguousarray(cube, dtype=np.complex128)
    if c.ndim != 3:
        raise ValueError("cube must be [planes][ny][nx]")
    check(_lib.load().wsg_write_cube_dump(c.ctypes.data, c.shape[0], c.shape[1], c.shape[2],
                                          float(scale), _b(real_path), _b(img_path)))


def plan_dump_cube(plan, cube, real_path, img_path, scale: float = 1.0) -> None:
    """The same dump from a cube resident on ``plan``'s device (a torch tensor)."""
    plan._sync_stream()
    check(plan.lib.wsg_plan_dump_cube(plan._h, cube.data_ptr(), float(scale), _b(real_path),
                                      _b(img_path)))


def write_image_dump(image_real: np.ndarray, image_imag: np.ndarray, real_path, img_path) -> None:
    re = np.ascontiguousarray(image_real, dtype=np.float64)
    im = np.ascontiguousarray(image_imag, dtype=np.float64)
    if re.size != im.size:
        raise ValueError("real and imaginary images differ in size")
    check(_lib.load().wsg_write_image_dump(re.ctypes.data, im.ctypes.data, re.size, _b(real_path),
                                           _b(img_path)))


def write_timings(path, seconds) -> None:
    s = (ctypes.c_double * 7)(*[float(x) for x in seconds])
    check(_lib.load().wsg_write_timings(_b(path), s))


def read_dump(real_path, img_path, shape) -> np.ndarray:
    """Two float64 dump files -> one complex128 array of ``shape``."""
    re = np.fromfile(real_path, dtype=np.float64)
    im = np.fromfile(img_path, dtype=np.float64)
    return (re + 1j * im).reshape(shape)


def run(paramfile, *, write_data: bool = False, write_image: bool = False,
        precision="fp64", outdir="", write_timings: bool = True, verbose: bool = False) -> dict:
    """The reference's main() on the current CUDA device -> report dict."""
    lib = _lib.load()
    o = _lib.RunOptions()
    lib.wsg_run_options_default(ctypes.byref(o))
    o.precision = {"fp64": WSG_FP64, "fp32c": WSG_FP32C}.get(precision, precision)
    o.write_data, o.write_image = int(write_data), int(write_image)
    o.write_timings, o.verbose = int(write_timings), int(verbose)
    o.outdir = os.fsencode(str(outdir))
    r = _lib.RunReport()
    check(lib.wsg_run_paramfile(_b(paramfile), ctypes.byref(o), ctypes.byref(r)))
    return {f: getattr(r, f) for f, _ in _lib.RunReport._fields_}


def write_dataset(directory, *, uu, vv, ww, weights, vis_real, vis_img, freq_per_chan: int,
                  polarisations: int, ntimes: int = 0, dt: float = 0.0, thours: float = 0.0,
                  baselines: int = 0, uvmin: float, uvmax: float, wmin: float, wmax: float,
                  names: dict | None = None) -> dict:
    """Write arrays as a reference dataset directory; returns the file names.

    meta.txt lists Nmeasures = len(uu): the reader drops the last 1000 of
    them, so pass 1000 rows more than are to be gridded."""
    names = dict(ufile="ucoord.bin", vfile="vcoord.bin", wfile="wcoord.bin",
                 weightsfile="weights.bin", visrealfile="visibilities_real.bin",
                 visimgfile="visibilities_img.bin", metafile="meta.txt", **(names or {}))
    os.makedirs(directory, exist_ok=True)
    n = len(uu)
    for key, arr, dt_ in (("ufile", uu, np.float64), ("vfile", vv, np.float64),
                          ("wfile", ww, np.float64), ("weightsfile", weights, np.float32),
                          ("visrealfile", vis_real, np.float32),
                          ("visimgfile", vis_img, np.float32)):
        np.ascontiguousarray(arr, dtype=dt_).tofile(os.path.join(directory, names[key]))
    nvis = n * freq_per_chan * polarisations
    with open(os.path.join(directory, names["metafile"]), "w") as f:
        f.write(f"{n}\n{nvis}\n{freq_per_chan}\n{polarisations}\n{ntimes}\n{dt!r}\n{thours!r}\n"
                f"{baselines}\n{uvmin!r}\n{uvmax!r}\n{wmin!r}\n{wmax!r}\n")
    return names


__all__ = ["read_parameter_file", "read_metadata", "partition_measurements", "read_measurements",
           "reference_resolution", "write_cube_dump", "plan_dump_cube", "write_image_dump",
           "write_timings", "read_dump", "run", "write_dataset", "META_FIELDS",
           "WSG_DROPPED_ROWS"]
