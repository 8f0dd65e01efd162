"""Writes the reference-format fixtures in tests/golden/binms/ and records what
the reference's own reader makes of them.

Run from anywhere in the container that holds the reference tree:

    python tests/golden/make_binms_golden.py

1. Seeded small datasets in the reference's input layout (ds0: 1137 rows with
   2 channels x 2 polarisations; ds1: 1050 rows, 1 x 1; short: value files cut
   short; edges: rows on and around v-slab edges) and parameter files that
   exercise the reference's parsing rules.
2. oracle/_ref/refio (the reference's init.c, allvars.c and gridding.c) reads
   each (parameter file, dataset, rank, size) case and sectors the rank's rows
   into nsectors = size v-slabs; its parameters, meta values after the
   partition, startrow, a SHA-256 of every array it read, histo_send and a
   SHA-256 of the concatenated slab lists go to expected.json.
3. One single-rank case runs the reference's gridding loop and grid dump
   writer too; the two dump files are kept in ref_grid/.
tests/test_binms.py checks the library and the restatements against these
records, so the checks need neither the reference nor refio.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "binms")
sys.path.insert(0, ROOT)

from oracle import binms_oracle as B  # noqa: E402
from oracle import build as oracle_build  # noqa: E402

PARAMFILE = """ndatasets              2
Datapath1              ds0/
Datapath2              ds1/
num_threads            2
w_support              7
grid_size_x            64
grid_size_y            64
num_w_planes           4
ufile\t\t       ucoord.bin
vfile    \t       vcoord.bin
wfile                  wcoord.bin
weightsfile\t       weights.bin
visrealfile            visibilities_real.bin
visimgfile             visibilities_img.bin
metafile               meta.txt
outfile                grid.txt
outfile1\t       coords.txt
outfile2\t       grid_real.bin
outfile3 \t       grid_img.bin
fftfile\t\t       fft.txt
fftfile2\t       fft_real.bin
fftfile3\t       fft_img.bin
logfile                run.log
extension              .txt
timingfile             timings.dat
verbose_level\t       1
"""

# ndatasets after the directories (so Datapath2 is not taken), a repeated
# key, keys and values on one line, and a trailing key without a value
PARAMFILE_QUIRKS = """Datapath1 ds0/ Datapath2 ds1/ ndatasets 2
num_threads 4 w_support 9 w_support 5 grid_size_x 32 grid_size_y 48 num_w_planes 2
ufile ucoord.bin vfile vcoord.bin wfile wcoord.bin weightsfile weights.bin
visrealfile visibilities_real.bin visimgfile visibilities_img.bin metafile meta.txt
outfile2 g_re.bin outfile3 g_im.bin fftfile2 f_re.bin fftfile3 f_im.bin
timingfile t.dat verbose_level 7 extension
"""

PARAMFILE_SHORT = PARAMFILE.replace("ndatasets              2", "ndatasets              1") \
                           .replace("ds0/", "short/")

# one rank, one thread (a deterministic sum), a 32 x 32 x 4 grid
PARAMFILE_GRID = PARAMFILE.replace("ndatasets              2", "ndatasets              1") \
                          .replace("num_threads            2", "num_threads            1") \
                          .replace("grid_size_x            64", "grid_size_x            32") \
                          .replace("grid_size_y            64", "grid_size_y            32")

PARAMFILE_EDGES = PARAMFILE.replace("ndatasets              2", "ndatasets              1") \
                           .replace("ds0/", "edges/")


def edge_rows():
    """v values on, just inside and just outside the slab edges and the
    w_supporth bands of a 64-row grid split into 1, 2, 4 and 8 slabs
    (w_support 7: w_supporth = 3/64)."""
    v = [0.0, 5e-324, 0.25, 0.5, 0.75, np.nextafter(1.0, 0.0)]
    for k in range(1, 8):
        e = k / 8.0
        for d in (0.0, 3 / 64, -3 / 64, 2 / 64, -2 / 64):
            x = e + d
            v += [x, np.nextafter(x, 0.0), np.nextafter(x, 1.0)]
    return np.array([x for x in v if 0.0 <= x < 1.0], dtype=np.float64)


def _dataset(directory, n, nf, npol, seed, meta_text_fn, cut=None):
    rng = np.random.default_rng(seed)
    os.makedirs(directory, exist_ok=True)
    arrays = {
        "ucoord.bin": rng.random(n),
        "vcoord.bin": rng.random(n),
        "wcoord.bin": rng.random(n),
        "weights.bin": rng.random(n * npol).astype(np.float32),
        "visibilities_real.bin": rng.standard_normal(n * nf * npol).astype(np.float32),
        "visibilities_img.bin": rng.standard_normal(n * nf * npol).astype(np.float32),
    }
    for name, a in arrays.items():
        b = a.tobytes()
        if cut and name in cut:
            b = b[:cut[name]]
        with open(os.path.join(directory, name), "wb") as f:
            f.write(b)
    with open(os.path.join(directory, "meta.txt"), "w") as f:
        f.write(meta_text_fn(n, nf, npol))


def _sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> int:
    if oracle_build.build_refio() is None:
        print("the reference tree is needed to build oracle/_ref/refio", file=sys.stderr)
        return 1
    os.makedirs(OUT, exist_ok=True)
    # meta.txt as the reference's converter writes it: one value per line;
    # ds1 uses tabs, an exponent and a negative uvmin to exercise the scanner
    _dataset(os.path.join(OUT, "ds0"), 1137, 2, 2, 11,
             lambda n, nf, p: f"{n}\n{n * nf * p}\n{nf}\n{p}\n379\n10.0\n1.05\n3\n"
                              f"-2345.75\n2987.5\n-612.25\n640.5\n")
    _dataset(os.path.join(OUT, "ds1"), 1050, 1, 1, 12,
             lambda n, nf, p: f"{n}\t{n * nf * p}\t{nf}\t{p}\t 1050 2.5e0 0.729 1\n"
                              f"-1.5e3 1499.9\n-3.25e2\t+4.0e2\n")
    # rows that are 1000 + 40, but the value files hold only 30 rows
    _dataset(os.path.join(OUT, "short"), 1040, 1, 2, 13,
             lambda n, nf, p: f"{n}\n{n * nf * p}\n{nf}\n{p}\n0\n1.0\n1.0\n1\n-100.0\n100.0\n"
                              f"-10.0\n10.0\n",
             cut={"visibilities_real.bin": 30 * 2 * 4, "visibilities_img.bin": 30 * 2 * 4})
    ev = edge_rows()
    _dataset(os.path.join(OUT, "edges"), len(ev) + 1000, 1, 1, 14,
             lambda n, nf, p: f"{n}\n{n * nf * p}\n{nf}\n{p}\n0\n1.0\n1.0\n1\n-100.0\n"
                              f"100.0\n-10.0\n10.0\n")
    vfull = np.fromfile(os.path.join(OUT, "edges", "vcoord.bin"))
    vfull[:len(ev)] = ev
    vfull.tofile(os.path.join(OUT, "edges", "vcoord.bin"))
    for name, text in (("paramfile.txt", PARAMFILE), ("paramfile_quirks.txt", PARAMFILE_QUIRKS),
                       ("paramfile_short.txt", PARAMFILE_SHORT),
                       ("paramfile_grid.txt", PARAMFILE_GRID),
                       ("paramfile_edges.txt", PARAMFILE_EDGES)):
        with open(os.path.join(OUT, name), "w") as f:
            f.write(text)

    cases = [("paramfile.txt", 0, 0, 1), ("paramfile.txt", 0, 0, 3), ("paramfile.txt", 0, 1, 3),
             ("paramfile.txt", 0, 2, 3), ("paramfile.txt", 1, 0, 1), ("paramfile.txt", 1, 1, 2),
             ("paramfile.txt", 0, 3, 7), ("paramfile.txt", 0, 6, 7),
             ("paramfile_quirks.txt", 0, 0, 1), ("paramfile_short.txt", 0, 0, 1)]
    cases += [("paramfile_edges.txt", 0, r, sz) for sz in (1, 2, 4, 8) for r in range(sz)]
    expected = []
    with tempfile.TemporaryDirectory() as tmp:
        for k, (pf, ds, rank, size) in enumerate(cases):
            r = B.run_refio(pf, ds, rank, size, os.path.join(tmp, str(k)), cwd=OUT)
            if r is None or r["returncode"] != 0:
                print(f"refio failed on {pf} {ds} {rank} {size}: {r}", file=sys.stderr)
                return 1
            expected.append({
                "paramfile": pf, "dataset": ds, "rank": rank, "size": size,
                "params": r["params"], "meta": r["meta"],
                "sha256": {k2: _sha(v) for k2, v in r["arrays"].items()},
                "short_read": "an error occurred while reading file" in r["stdout"],
                "histo": [int(x) for x in r["histo"]],
                "sectors_sha256": _sha(np.concatenate(r["lists"]) if r["lists"] else
                                       np.zeros(0, np.int64)),
            })
        # the reference's single-rank gridding and grid dump
        r = B.run_refio("paramfile_grid.txt", 0, 0, 1, os.path.join(tmp, "grid"), cwd=OUT,
                        grid=True)
        if r is None or r["returncode"] != 0:
            print(f"refio grid failed: {r}", file=sys.stderr)
            return 1
        os.makedirs(os.path.join(OUT, "ref_grid"), exist_ok=True)
        for f in ("0grid_real.bin", "0grid_img.bin"):
            with open(os.path.join(r["outdir"], f), "rb") as src, \
                    open(os.path.join(OUT, "ref_grid", f), "wb") as dst:
                dst.write(src.read())
    with open(os.path.join(OUT, "expected.json"), "w") as f:
        json.dump(expected, f, indent=1, sort_keys=True)
    print(f"wrote {len(expected)} cases to {os.path.join(OUT, 'expected.json')}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
