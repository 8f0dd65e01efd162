"""The reference's files through the library (include/wstack_gb300_io.h), on CPU.

Reader: the library's parameter-file, meta-file and binary-file reader against
(1) tests/golden/binms/expected.json -- what the reference's own reader
(init.c, compiled into oracle/_ref/refio) read from the fixtures in
tests/golden/binms/, recorded by tests/golden/make_binms_golden.py -- and
(2) the NumPy restatement in oracle/binms_oracle.py, itself pinned to the same
records and, where refio is built, to refio run afresh.  All integer, byte and
array comparisons are exact.

Dumps: the grid / fft / image dump files and the timing line against the
restatement of gridding.c:428-438, fourier_transform.c:177-219 and
result.c:53-56, byte for byte.
"""
import ctypes
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

from lofar_gb300 import _lib, binms
from lofar_gb300._lib import WstackError
from oracle import binms_oracle as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "binms")
EXPECTED = json.load(open(os.path.join(GOLD, "expected.json")))
CASE_IDS = [f"{c['paramfile'][:-4]}-ds{c['dataset']}-r{c['rank']}of{c['size']}" for c in EXPECTED]
ARRAYS = ("uu", "vv", "ww", "weights", "vis_real", "vis_img")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from lofar_gb300 import build
        build.build()
    return _lib.load()


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _expected_params(case):
    """refio's params.txt -> (numbers, directories, names without the dataset prefix)."""
    p = case["params"]
    nums = {k: int(p[k]) for k in ("num_threads", "ndatasets", "grid_size_x", "grid_size_y",
                                   "num_w_planes", "w_support", "verbose_level")}
    dirs = {int(k[len("datapath"):]): v for k, v in p.items() if k.startswith("datapath")}
    pre = str(case["dataset"])
    names = {}
    for k in B.NAME_KEYS:
        v = p.get(k, "")
        if k.startswith(("outfile", "fftfile")) or k in ("logfile", "extension", "timingfile"):
            assert v.startswith(pre)   # op_filename, init.c:67-121
            v = v[len(pre):]
        names[k] = v
    return nums, dirs, names


def _read_with_library(lib, case):
    """The reference's init() sequence through the C ABI; returns
    (params dict, meta after the partition, startrow, arrays, read status)."""
    prm = _lib.Params()
    assert lib.wsg_read_parameter_file(case["paramfile"].encode(), ctypes.byref(prm)) == 0
    ds = case["dataset"]
    meta = _lib.Metadata()
    path = prm.datapath[ds].value + prm.metafile
    assert lib.wsg_read_metadata(path, ctypes.byref(meta)) == 0
    start = ctypes.c_long()
    assert lib.wsg_partition_measurements(ctypes.byref(meta), case["rank"], case["size"],
                                          ctypes.byref(start)) == 0
    n, nw, nv = meta.Nmeasures, meta.Nweights, meta.Nvis
    arrs = {"uu": np.full(n, 7.0), "vv": np.full(n, 7.0), "ww": np.full(n, 7.0),
            "weights": np.full(nw, 7, np.float32), "vis_real": np.full(nv, 7, np.float32),
            "vis_img": np.full(nv, 7, np.float32)}
    st = lib.wsg_read_measurements(ctypes.byref(prm), ds, ctypes.byref(meta), start.value,
                                   *[arrs[k].ctypes.data for k in ARRAYS])
    return binms._params_dict(prm), binms._meta_dict(meta), start.value, arrs, st


@pytest.mark.parametrize("case", EXPECTED, ids=CASE_IDS)
def test_library_reader_matches_the_reference_reader(lib, case, monkeypatch):
    monkeypatch.chdir(GOLD)
    params, meta, start, arrs, st = _read_with_library(lib, case)
    nums, dirs, names = _expected_params(case)
    for k, v in nums.items():
        assert params[k] == v, k
    assert {i: d for i, d in enumerate(params["datapath"]) if d} == dirs
    for k, v in names.items():
        assert params[k] == v, k
    em = case["meta"]
    for k in ("Nmeasures", "Nvis", "Nweights", "freq_per_chan", "polarisations", "Ntimes",
              "baselines"):
        assert meta[k] == em[k], k
    for k in ("dt", "thours", "uvmin", "uvmax", "wmin", "wmax"):
        assert meta[k] == em[k], k
    assert start == em["startrow"]
    for k in ARRAYS:
        assert _sha(arrs[k]) == case["sha256"][k], k
    # the reference prints and carries on with zero-filled buffers; the library
    # zero-fills the same way and reports the short file
    if case["short_read"]:
        assert st == _lib.WSG_ERR_IO
        assert b"an error occurred while reading file" in lib.wstack_gb300_last_error_string()
    else:
        assert st == 0


@pytest.mark.parametrize("case", EXPECTED, ids=CASE_IDS)
def test_restatement_matches_the_reference_reader(case, monkeypatch):
    """Pins oracle/binms_oracle.py to the recorded reference results."""
    monkeypatch.chdir(GOLD)
    p = B.parse_parameter_file(open(case["paramfile"]).read())
    nums, dirs, names = _expected_params(case)
    for k, v in nums.items():
        assert p[k] == v, k
    assert {i: d for i, d in enumerate(p["datapath"]) if d} == dirs
    for k, v in names.items():
        assert p[k] == v, k
    d = p["datapath"][case["dataset"]]
    meta, start = B.partition(B.parse_metadata(open(d + p["metafile"]).read()), case["rank"],
                              case["size"])
    assert start == case["meta"]["startrow"]
    for k in ("Nmeasures", "Nvis", "Nweights", "dt", "uvmin", "wmax"):
        assert meta[k] == case["meta"][k]
    if not case["short_read"]:
        got = B.read_measurements(d, p, meta, start)
        for k in ARRAYS:
            assert _sha(got[k]) == case["sha256"][k], k


def _case_rows(case):
    """The rows the case's rank reads, through the restatement."""
    p = B.parse_parameter_file(open(os.path.join(GOLD, case["paramfile"])).read())
    d = os.path.join(GOLD, p["datapath"][case["dataset"]])
    meta, start = B.partition(B.parse_metadata(open(os.path.join(d, p["metafile"])).read()),
                              case["rank"], case["size"])
    return p, B.read_measurements(d + "/", p, meta, start)


def _sector_geometry(p, size):
    dx = 1.0 / p["grid_size_x"]
    return size, p["grid_size_y"] // size, dx, float((p["w_support"] - 1) // 2) * dx


@pytest.mark.parametrize("case", [c for c in EXPECTED if not c["short_read"]],
                         ids=[i for i, c in zip(CASE_IDS, EXPECTED) if not c["short_read"]])
def test_sector_restatement_matches_the_reference(case):
    """initialize_array (gridding.c:35-86) restated, against the reference's
    histo_send and lists for nsectors = ranks, edge rows included."""
    p, rows = _case_rows(case)
    histo, lists = B.initialize_array(rows["vv"], *_sector_geometry(p, case["size"]))
    assert histo.tolist() == case["histo"]
    assert _sha(np.concatenate(lists)) == case["sectors_sha256"]


def test_reference_grid_dump_pins_the_oracle_and_the_writer(lib, tmp_path):
    """The reference's own single-rank gridding and grid dump (ref_grid/,
    num_threads 1) equal, bit for bit, the oracle gridding the slab's rows in
    the reference's order (reverse list order) and the library's writer
    dumping that grid."""
    from oracle import oracle as O
    p = B.parse_parameter_file(open(os.path.join(GOLD, "paramfile_grid.txt")).read())
    d = os.path.join(GOLD, p["datapath"][0])
    meta, start = B.partition(B.parse_metadata(open(os.path.join(d, p["metafile"])).read()))
    rows = B.read_measurements(d, p, meta, start)
    nx, ny, P, S = p["grid_size_x"], p["grid_size_y"], p["num_w_planes"], p["w_support"]
    nf, npol = meta["freq_per_chan"], meta["polarisations"]
    histo, lists = B.initialize_array(rows["vv"], *_sector_geometry(p, 1))
    c = B.sector_compose(lists[0], 0, ny, 1.0 / nx, rows["uu"], rows["vv"], rows["ww"],
                         rows["weights"], rows["vis_real"], rows["vis_img"], nf, npol)
    grid = O.wstack(c["uu"], c["vv"], c["ww"], c["vis_real"], c["vis_img"], c["weights"],
                    num_w_planes=P, freq_per_chan=nf, polarizations=npol, dx=1.0 / nx,
                    dw=1.0 / P, w_support=S, nx=nx, ny=ny, num_threads=1)
    ref_re = open(os.path.join(GOLD, "ref_grid", "0grid_real.bin"), "rb").read()
    ref_im = open(os.path.join(GOLD, "ref_grid", "0grid_img.bin"), "rb").read()
    cube = grid[..., 0] + 1j * grid[..., 1]
    binms.write_cube_dump(cube, tmp_path / "re.bin", tmp_path / "im.bin")
    assert (tmp_path / "re.bin").read_bytes() == ref_re
    assert (tmp_path / "im.bin").read_bytes() == ref_im


@pytest.mark.skipif(not os.path.exists(B.REFIO), reason="oracle/_ref/refio not built here")
@pytest.mark.parametrize("case", EXPECTED, ids=CASE_IDS)
def test_fixtures_still_match_a_fresh_reference_run(case, tmp_path):
    r = B.run_refio(case["paramfile"], case["dataset"], case["rank"], case["size"],
                    str(tmp_path), cwd=GOLD)
    assert r["returncode"] == 0
    assert r["params"] == case["params"]
    assert r["meta"] == case["meta"]
    for k in ARRAYS:
        assert _sha(r["arrays"][k]) == case["sha256"][k]
    assert r["histo"].tolist() == case["histo"]
    assert _sha(np.concatenate(r["lists"])) == case["sectors_sha256"]


@pytest.mark.skipif(not os.path.exists(B.REFIO), reason="oracle/_ref/refio not built here")
def test_reference_grid_fixture_still_matches_a_fresh_run(tmp_path):
    r = B.run_refio("paramfile_grid.txt", 0, 0, 1, str(tmp_path), cwd=GOLD, grid=True)
    assert r["returncode"] == 0
    for f in ("0grid_real.bin", "0grid_img.bin"):
        assert (tmp_path / f).read_bytes() == open(os.path.join(GOLD, "ref_grid", f), "rb").read()


def test_python_front_end_reads_a_dataset(lib, monkeypatch):
    monkeypatch.chdir(GOLD)
    p = binms.read_parameter_file("paramfile.txt")
    assert p["datapath"] == ["ds0/", "ds1/"] and p["ndatasets"] == 2
    meta = binms.read_metadata(p["datapath"][1] + p["metafile"])
    assert meta["Nmeasures"] == 1050 and meta["uvmin"] == -1500.0 and meta["wmax"] == 400.0
    m, start = binms.partition_measurements(meta, 1, 2)
    assert (m["Nmeasures"], start) == (25, 25)
    got = binms.read_measurements(p, 1, m, start)
    ref = B.read_measurements("ds1/", B.parse_parameter_file(open("paramfile.txt").read()), m, start)
    for k in ARRAYS:
        assert np.array_equal(got[k], ref[k])


# --------------------------------------------------------------------------
# errors: the reference exits or carries on; the library returns a status
# --------------------------------------------------------------------------

def test_reader_errors(lib, tmp_path):
    with pytest.raises(WstackError, match="error opening paramfile"):
        binms.read_parameter_file(tmp_path / "missing.txt")
    with pytest.raises(WstackError, match="error opening meta file"):
        binms.read_metadata(tmp_path / "missing.txt")
    (tmp_path / "bad_meta.txt").write_text("2000 2000 1 1 10 1.0 x\n")
    with pytest.raises(WstackError, match="field 7 .thours. is not a number"):
        binms.read_metadata(tmp_path / "bad_meta.txt")
    (tmp_path / "short_meta.txt").write_text("2000 2000 1 1\n")
    with pytest.raises(WstackError, match="field 5"):
        binms.read_metadata(tmp_path / "short_meta.txt")
    (tmp_path / "long.txt").write_text("ufile " + "a" * 300 + "\n")
    with pytest.raises(WstackError, match="ufile longer than"):
        binms.read_parameter_file(tmp_path / "long.txt")
    meta = dict(Nmeasures=999, freq_per_chan=1, polarisations=1)
    with pytest.raises(WstackError, match="fewer than the 1000 dropped"):
        binms.partition_measurements(meta)
    with pytest.raises(WstackError, match="outside"):
        binms.partition_measurements(dict(meta, Nmeasures=5000), rank=2, size=2)
    p = {"datapath": [str(tmp_path) + "/"], "ufile": "nope.bin", "vfile": "nope.bin",
         "wfile": "nope.bin", "weightsfile": "nope.bin", "visrealfile": "nope.bin",
         "visimgfile": "nope.bin"}
    m = dict(Nmeasures=4, Nvis=4, Nweights=4, freq_per_chan=1, polarisations=1)
    with pytest.raises(WstackError, match="error opening ucoord file"):
        binms.read_measurements(p, 0, m, 0)


def test_metadata_scanner_follows_scanf(lib, tmp_path):
    (tmp_path / "m.txt").write_text("+2000\t9 1 1 0 1e0 .5\n2 -3.5 7 -1 0x10\n")
    m = binms.read_metadata(tmp_path / "m.txt")
    assert m["Nmeasures"] == 2000 and m["Nvis"] == 9 and m["dt"] == 1.0 and m["thours"] == 0.5
    assert m["uvmin"] == -3.5 and m["wmin"] == -1.0 and m["wmax"] == 16.0   # %lf reads hex
    # %ld stops at the '.', and the next %ld cannot start there
    (tmp_path / "m.txt").write_text("1500.5 9 1 1 0 1 1 2 -3.5 7 -1 1\n")
    with pytest.raises(WstackError, match="field 2 .Nvis. is not an integer"):
        binms.read_metadata(tmp_path / "m.txt")


@pytest.mark.parametrize("uvmin,uvmax", [(-2345.75, 2987.5), (-1.5e3, 1499.9), (0.4, -0.9),
                                         (-7.99, 7.5), (12.0, -12.0)])
def test_reference_resolution_truncates_like_int_abs(lib, uvmin, uvmax):
    assert binms.reference_resolution(uvmin, uvmax) == B.resolution(uvmin, uvmax)
    with pytest.raises(WstackError):
        binms.reference_resolution(1e12, 1.0)


# --------------------------------------------------------------------------
# dumps and the timing line, byte for byte
# --------------------------------------------------------------------------

def test_cube_dump_bytes(lib, tmp_path):
    rng = np.random.default_rng(5)
    cube = rng.standard_normal((3, 40, 24)) + 1j * rng.standard_normal((3, 40, 24))
    for scale in (1.0, 1.0 / (40 * 24)):
        binms.write_cube_dump(cube, tmp_path / "re.bin", tmp_path / "im.bin", scale=scale)
        want_re, want_im = B.cube_dump(cube, scale)
        assert (tmp_path / "re.bin").read_bytes() == want_re
        assert (tmp_path / "im.bin").read_bytes() == want_im
    got = binms.read_dump(tmp_path / "re.bin", tmp_path / "im.bin", cube.shape)
    assert np.array_equal(got, cube * (1.0 / (40 * 24)))


def test_cube_dump_spans_several_chunks(lib, tmp_path):
    # 2^20 elements per chunk in the host writer: 1.5 chunks here
    cube = (np.arange(3 << 19, dtype=np.float64) - 7.25j).reshape(6, 512, 512)
    binms.write_cube_dump(cube, tmp_path / "re.bin", tmp_path / "im.bin")
    want_re, want_im = B.cube_dump(cube)
    assert (tmp_path / "re.bin").read_bytes() == want_re
    assert (tmp_path / "im.bin").read_bytes() == want_im


def test_image_dump_and_timings_bytes(lib, tmp_path):
    rng = np.random.default_rng(6)
    re, im = rng.standard_normal((2, 33, 17))
    re[3, 4] = np.nan   # NaN pixels are written as they are
    binms.write_image_dump(re, im, tmp_path / "f_re.bin", tmp_path / "f_im.bin")
    want_re, want_im = B.image_dump(re, im)
    assert (tmp_path / "f_re.bin").read_bytes() == want_re
    assert (tmp_path / "f_im.bin").read_bytes() == want_im
    t = [0.125, 1.5, 2.0, 0.0, 3.25, 4.0, 1e-7]
    binms.write_timings(tmp_path / "t.dat", t)
    assert (tmp_path / "t.dat").read_text() == B.timings_line(t)


def test_dump_errors(lib, tmp_path):
    with pytest.raises(WstackError, match="cannot open"):
        binms.write_cube_dump(np.zeros((1, 2, 2), complex), tmp_path / "no" / "re.bin",
                              tmp_path / "im.bin")
    with pytest.raises(WstackError, match="cannot open"):
        binms.write_timings(tmp_path / "no" / "t.dat", [0] * 7)


def test_write_dataset_round_trip(lib, tmp_path):
    rng = np.random.default_rng(8)
    n, nf, npol = 1200, 3, 2
    arrs = dict(uu=rng.random(n), vv=rng.random(n), ww=rng.random(n),
                weights=rng.random(n * npol).astype(np.float32),
                vis_real=rng.standard_normal(n * nf * npol).astype(np.float32),
                vis_img=rng.standard_normal(n * nf * npol).astype(np.float32))
    names = binms.write_dataset(tmp_path / "ds", freq_per_chan=nf, polarisations=npol,
                                uvmin=-10.5, uvmax=11.25, wmin=-3.0, wmax=4.0, **arrs)
    meta = binms.read_metadata(tmp_path / "ds" / names["metafile"])
    assert meta["Nmeasures"] == n and meta["uvmax"] == 11.25
    m, start = binms.partition_measurements(meta)
    params = dict(names, datapath=[str(tmp_path / "ds") + "/"])
    got = binms.read_measurements(params, 0, m, start)
    keep = n - 1000
    assert np.array_equal(got["uu"], arrs["uu"][:keep])
    assert np.array_equal(got["weights"], arrs["weights"][:keep * npol])
    assert np.array_equal(got["vis_img"], arrs["vis_img"][:keep * nf * npol])


# --------------------------------------------------------------------------
# the driver and its executable fail loudly without a GPU
# --------------------------------------------------------------------------

def _no_gpu():
    try:
        import torch
        return not torch.cuda.is_available()
    except Exception:
        return True


@pytest.mark.skipif(not _no_gpu(), reason="checks the behaviour without a GPU")
def test_driver_reports_the_missing_gpu(lib, monkeypatch):
    monkeypatch.chdir(GOLD)
    with pytest.raises(WstackError) as e:
        binms.run("paramfile.txt")
    assert e.value.status in (_lib.WSG_ERR_CUDA, _lib.WSG_ERR_NOMEM)


def test_driver_argument_errors(lib, tmp_path):
    (tmp_path / "p.txt").write_text("num_threads 0\nndatasets 1\n")
    with pytest.raises(WstackError, match="number_of_OMP_Threads"):
        binms.run(tmp_path / "p.txt")
    (tmp_path / "p.txt").write_text("num_threads 1\nndatasets 101\n")
    with pytest.raises(WstackError, match="ndatasets 101"):
        binms.run(tmp_path / "p.txt")
    with pytest.raises(WstackError, match="invalid precision"):
        binms.run(tmp_path / "p.txt", precision=5)


def test_sector_argument_errors_need_no_gpu(lib):
    assert lib.wsg_sector_count(None, 10, 0, 8, 1 / 64, 3 / 64, None, None) == \
        _lib.WSG_ERR_UNSUPPORTED
    assert lib.wsg_sector_count(None, 10, 1024, 8, 1 / 64, 3 / 64, None, None) == \
        _lib.WSG_ERR_UNSUPPORTED
    assert lib.wsg_sector_lists(None, 10, 4, 0, 1 / 64, 3 / 64, None, None, 0, None) == \
        _lib.WSG_ERR_ARG
    assert lib.wsg_sector_lists(None, 10, 4, 16, -1.0, 3 / 64, None, None, 0, None) == \
        _lib.WSG_ERR_ARG
    assert lib.wsg_sector_gather(None, 5, 0, 16, 1 / 64, 1, 1, *([None] * 12), None) == \
        _lib.WSG_ERR_ARG
    assert lib.wsg_initialize_array(None, 10, 4, 16, 1 / 64, 3 / 64, None, None) == \
        _lib.WSG_ERR_ARG


def test_runner_executable_usage(lib):
    from lofar_gb300 import build
    if not os.path.exists(build.RUNNER):
        build.build()
    r = subprocess.run([build.RUNNER], capture_output=True, text=True)
    assert r.returncode == 1 and "Parameter file is not given" in r.stderr
    r = subprocess.run([build.RUNNER, "/nonexistent/paramfile"], capture_output=True, text=True)
    assert r.returncode == 1 and "error opening paramfile" in r.stderr
