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


def initialize_array(vv: np.ndarray, nsectors: int, yaxis: int, dx: float,
                     w_supporth: float) -> tuple[np.ndarray, list]:
    """gridding.c:35-86: histo_send[nsectors+1] and the per-slab row lists.

    binphi = (int)(vv*nsectors); a row also joins slab binphi+1 (binphi-1)
    when its distance to that edge, (double)((binphi+1)*yaxis)*dx - vv
    (vv - (double)(binphi*yaxis)*dx), is in [0, w_supporth) (and binphi > 0
    for the lower edge).  Lists are in increasing row order (the second pass
    appends in row order).  NumPy float64 arithmetic is IEEE with one rounding
    per operation, as the reference's C."""
    vv = np.asarray(vv, dtype=np.float64)
    x = vv * float(nsectors)
    if not np.all((x > -1.0) & (x < nsectors + 1.0)):
        raise ValueError("a row's slab index is outside [0, nsectors]")
    b = np.trunc(x).astype(np.int64)
    updist = ((b + 1) * yaxis).astype(np.float64) * dx - vv
    downdist = vv - (b * yaxis).astype(np.float64) * dx
    up = (updist < w_supporth) & (updist >= 0.0)
    down = (downdist < w_supporth) & (b > 0) & (downdist >= 0.0)
    if np.any(up & (b + 1 > nsectors)):
        raise ValueError("a row joins slab nsectors + 1")
    rows = np.arange(vv.shape[0], dtype=np.int64)
    # (slab, row) pairs of every membership, ordered by slab then row
    keys = np.concatenate([b, b[up] + 1, b[down] - 1])
    who = np.concatenate([rows, rows[up], rows[down]])
    order = np.lexsort((who, keys))
    histo = np.bincount(keys, minlength=nsectors + 1).astype(np.int64)
    lists = np.split(who[order], np.cumsum(histo)[:-1])
    return histo, lists


def sector_compose(lst: np.ndarray, isector: int, yaxis: int, dx: float, uu, vv, ww, weights,
                   vis_real, vis_img, nf: int, npol: int) -> dict:
    """gridding.c:193-211: the slab's rows in reverse list order, vv shifted
    by isector*shift with shift = (double)(dx*yaxis)."""
    r = np.asarray(lst, dtype=np.int64)[::-1]
    shift = dx * float(yaxis)
    return {"uu": np.asarray(uu)[r], "vv": np.asarray(vv)[r] - float(isector) * shift,
            "ww": np.asarray(ww)[r],
            "weights": np.asarray(weights).reshape(-1, npol)[r].reshape(-1),
            "vis_real": np.asarray(vis_real).reshape(-1, nf * npol)[r].reshape(-1),
            "vis_img": np.asarray(vis_img).reshape(-1, nf * npol)[r].reshape(-1)}


def run_refio(paramfile: str, dataset: int, rank: int, size: int, outdir: str,
              cwd: str | None = None, grid: bool = False) -> dict | None:
    """Run the reference's reader and sectoring (oracle/_ref/refio), and with
    ``grid`` its single-rank gridding and grid dump; None when it is not built."""
    if not os.path.exists(REFIO):
        return None
    os.makedirs(outdir, exist_ok=True)
    outdir = os.path.abspath(outdir)
    cmd = [REFIO, paramfile, str(dataset), str(rank), str(size), outdir] + (["grid"] if grid else [])
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=cwd)
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
    histo = np.array([int(x) for x in open(os.path.join(outdir, "histo.txt")).read().split()],
                     dtype=np.int64)
    flat = np.fromfile(os.path.join(outdir, "sectors.bin"), dtype=np.int64)
    lists = np.split(flat, np.cumsum(histo)[:-1]) if histo.size else []
    return {"returncode": 0, "stdout": r.stdout, "params": params, "meta": meta,
            "arrays": arrays, "histo": histo, "lists": lists, "outdir": outdir}
