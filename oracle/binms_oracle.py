"""NumPy restatement of the reference's file formats (test infrastructure only).

The checker for lofar_gb300's reader, dumps and driver
(include/wstack_gb300_io.h).  Each function restates one piece of the
reference; tests/test_binms.py pins these restatements against the
reference's own reader compiled into oracle/_ref/refio (when the reference
tree is present) and against the committed fixtures in tests/golden/binms/.
Nothing in the product imports this module.
"""
from __future__ import annotations

import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFIO = os.path.join(HERE, "_ref", "refio")

NAME_KEYS = ("ufile", "vfile", "wfile", "weightsfile", "visrealfile", "visimgfile", "metafile",
             "outfile", "outfile1", "outfile2", "outfile3", "fftfile", "fftfile2", "fftfile3",
             "logfile", "extension", "timingfile")
INT_KEYS = ("num_threads", "ndatasets", "grid_size_x", "grid_size_y", "num_w_planes", "w_support")
META_FIELDS = ("Nmeasures", "Nvis", "freq_per_chan", "polarisations", "Ntimes", "dt", "thours",
               "baselines", "uvmin", "uvmax", "wmin", "wmax")
META_INT = {"Nmeasures", "Nvis", "freq_per_chan", "polarisations", "Ntimes", "baselines"}


def _atoi(s: str) -> int:
    m = re.match(r"\s*([+-]?\d+)", s)
    return int(m.group(1)) if m else 0


def parse_parameter_file(text: str) -> dict:
    """init.c:124-250: (key, value) token pairs; see the library's header for the rules."""
    toks = text.split()
    p = {k: 0 for k in INT_KEYS}
    p.update({k: "" for k in NAME_KEYS})
    p["verbose_level"] = 0
    paths: dict[int, str] = {}
    i = 1                                    # init.c:130
    value = ""
    for t in range(0, len(toks), 2):
        key = toks[t]
        if t + 1 < len(toks):
            value = toks[t + 1]
        if key in INT_KEYS and key != "ndatasets":
            p[key] = _atoi(value)
        if key == "Datapath1":               # init.c:137-141
            paths[0] = value
            i += 1
        if key == "ndatasets":
            p["ndatasets"] = _atoi(value)
        if key in NAME_KEYS:
            p[key] = value
        if key == "verbose_level":           # init.c:233-236 converts the key
            p["verbose_level"] = _atoi(key)
        if p["ndatasets"] > 1 and key == f"Datapath{i}":   # init.c:238-247
            paths[i - 1] = value
            i += 1
    p["datapath"] = [paths.get(k, "") for k in range(i - 1)]
    return p


def parse_metadata(text: str) -> dict:
    """init.c:278-307: 12 numbers, %ld or %lf by field."""
    toks = text.split()
    if len(toks) < 12:
        raise ValueError("meta file has fewer than 12 fields")
    m = {f: (int(toks[k]) if f in META_INT else float(toks[k])) for k, f in enumerate(META_FIELDS)}
    m["Nweights"] = 0
    return m


def partition(meta: dict, rank: int = 0, size: int = 1) -> tuple[dict, int]:
    """init.c:311-343: drop the last 1000 rows, split contiguously, last rank takes the rest."""
    m = dict(meta)
    total = m["Nmeasures"] - 1000
    per, rem = total // size, total % size
    start = rank * per
    if rank == size - 1:
        per += rem
    m["Nmeasures"] = per
    m["Nvis"] = per * m["freq_per_chan"] * m["polarisations"]
    m["Nweights"] = per * m["polarisations"]
    return m, start


def read_measurements(directory: str, params: dict, meta: dict, startrow: int) -> dict:
    """init.c:387-501: float64 uvw rows, float32 [m][p] weights, float32 [m][f][p] values."""
    f, p = meta["freq_per_chan"], meta["polarisations"]
    n = meta["Nmeasures"]

    def rd(key, dtype, per_row, count):
        return np.fromfile(directory + params[key], dtype=dtype, count=count,
                           offset=startrow * per_row * np.dtype(dtype).itemsize)
    return {"uu": rd("ufile", np.float64, 1, n), "vv": rd("vfile", np.float64, 1, n),
            "ww": rd("wfile", np.float64, 1, n), "weights": rd("weightsfile", np.float32, p, n * p),
            "vis_real": rd("visrealfile", np.float32, f * p, n * f * p),
            "vis_img": rd("visimgfile", np.float32, f * p, n * f * p)}


def resolution(uvmin: float, uvmax: float) -> float:
    """gridding.c:160 with C's int abs()."""
    a, b = abs(int(uvmin)), abs(int(uvmax))
    m = max(a, b)
    return 1.0 / m if m else float("inf")


def cube_dump(cube: np.ndarray, scale: float = 1.0) -> tuple[bytes, bytes]:
    """gridding.c:428-438 / fourier_transform.c:84-139 with one rank: the real
    and the imaginary parts of the [plane][v][u] cube as float64, in order."""
    c = np.asarray(cube, dtype=np.complex128)
    return ((c.real * scale).astype("<f8").tobytes(), (c.imag * scale).astype("<f8").tobytes())


def image_dump(image_real: np.ndarray, image_imag: np.ndarray) -> tuple[bytes, bytes]:
    """fourier_transform.c:177-219: the [v][u] image parts as float64."""
    return (np.asarray(image_real, "<f8").tobytes(), np.asarray(image_imag, "<f8").tobytes())


def timings_line(seconds) -> str:
    """result.c:53-56."""
    return "%f %f %f %f %f %f %f\n" % tuple(seconds)


def run_refio(paramfile: str, dataset: int, rank: int, size: int, outdir: str,
              cwd: str | None = None) -> dict | None:
    """Run the reference's reader (oracle/_ref/refio); None when it is not built."""
    if not os.path.exists(REFIO):
        return None
    os.makedirs(outdir, exist_ok=True)
    r = subprocess.run([REFIO, paramfile, str(dataset), str(rank), str(size), outdir],
                       capture_output=True, text=True, cwd=cwd)
    if r.returncode != 0:
        return {"returncode": r.returncode, "stdout": r.stdout, "stderr": r.stderr}
    params = {}
    for ln in open(os.path.join(outdir, "params.txt")).read().splitlines():
        k, _, v = ln.partition(" ")
        params[k] = v
    vals = open(os.path.join(outdir, "meta.txt")).read().split()
    names = ("Nmeasures", "Nvis", "Nweights", "freq_per_chan", "polarisations", "Ntimes", "dt",
             "thours", "baselines", "uvmin", "uvmax", "wmin", "wmax", "startrow")
    meta = {k: (float(v) if k in ("dt", "thours", "uvmin", "uvmax", "wmin", "wmax") else int(v))
            for k, v in zip(names, vals)}
    arrays = {k: np.fromfile(os.path.join(outdir, f), dtype=dt) for k, f, dt in (
        ("uu", "uu.bin", np.float64), ("vv", "vv.bin", np.float64), ("ww", "ww.bin", np.float64),
        ("weights", "weights.bin", np.float32), ("vis_real", "visreal.bin", np.float32),
        ("vis_img", "visimg.bin", np.float32))}
    return {"returncode": 0, "stdout": r.stdout, "params": params, "meta": meta,
            "arrays": arrays}
