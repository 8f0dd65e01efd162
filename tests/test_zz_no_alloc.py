"""wsg_grid_noalloc: gridding for callers that cannot allocate device memory.

Some callers of this library cannot call cudaMalloc while they grid -- a
real-time pipeline that reserves all device memory before observing, or a
host application that owns the device memory and lends its plug-ins only its
own buffers.  wsg_grid_noalloc serves them: its intermediates live in a fixed
static device array inside the library.  This test calls it through the C ABI
twice in a row on different batches (so stale scratch contents from the first
call must not leak into the second) and compares each result with the
allocating drop-in wstack() at the FP64 grid tolerance of the parity tests
(1e-12 normwise).  It also checks that the second call does not change the
device's free memory, and that oversized calls and host pointers are refused
with a clear error.  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _nrm_max(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_noalloc_grid_matches_wstack_on_two_calls(gpu):
    import torch

    import lofar_gb300 as L
    from lofar_gb300 import _lib, synth

    lib = _lib.load()
    L.set_precision("fp64")
    nx, ny, planes, support = 256, 192, 8, 7
    obs = synth.observe(n_stations=30, diameter_m=3000.0, hours=3.0, n_vis=300_000, sky_seed=6)
    batches = [slice(0, 180_000), slice(180_000, 300_000)]
    stream = torch.cuda.current_stream().cuda_stream
    grid = torch.full((planes, ny, nx, 2), 5.0, dtype=torch.float64, device="cuda")
    for call, sel in enumerate(batches):
        host = {k: np.ascontiguousarray(getattr(obs, k)[sel])
                for k in ("uu", "vv", "ww", "vis_real", "vis_img", "weight")}
        n = host["uu"].shape[0]
        ref = np.zeros((planes, ny, nx, 2))
        L.wstack(planes, n, 1, 1, host["uu"], host["vv"], host["ww"], host["vis_real"],
                 host["vis_img"], host["weight"], 1.0 / nx, 1.0 / planes, support, nx, ny, ref, 1)
        dev = {k: torch.as_tensor(v).cuda() for k, v in host.items()}
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = lib.wsg_grid_noalloc(planes, n, 1, 1, dev["uu"].data_ptr(), dev["vv"].data_ptr(),
                                  dev["ww"].data_ptr(), dev["vis_real"].data_ptr(),
                                  dev["vis_img"].data_ptr(), dev["weight"].data_ptr(),
                                  1.0 / nx, 1.0 / planes, support, nx, ny, grid.data_ptr(),
                                  ctypes.c_void_p(stream))
        assert st == _lib.WSG_OK, _lib.last_error()
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if call == 1:
            assert free_after == free_before
        assert _nrm_max(grid.cpu().numpy(), ref) <= 1e-12, call


def test_noalloc_refuses_what_it_cannot_hold(gpu):
    import torch

    from lofar_gb300 import _lib

    lib = _lib.load()
    n = 2_000_000  # 160 B per measurement: above the fixed 64 MiB array
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    f = torch.zeros(n, dtype=torch.float32, device="cuda")
    grid = torch.zeros((4, 64, 64, 2), dtype=torch.float64, device="cuda")
    st = lib.wsg_grid_noalloc(4, n, 1, 1, x.data_ptr(), x.data_ptr(), x.data_ptr(), f.data_ptr(),
                              f.data_ptr(), f.data_ptr(), 1 / 64, 0.25, 7, 64, 64, grid.data_ptr(),
                              None)
    assert st == _lib.WSG_ERR_CAPACITY
    assert "scratch" in _lib.last_error()[1]
    h = np.zeros(10)
    st = lib.wsg_grid_noalloc(4, 10, 1, 1, h.ctypes.data, h.ctypes.data, h.ctypes.data,
                              h.ctypes.data, h.ctypes.data, h.ctypes.data, 1 / 64, 0.25, 7, 64, 64,
                              grid.data_ptr(), None)
    assert st == _lib.WSG_ERR_ARG


def test_noalloc_folds_channels_and_polarisations_at_the_grid_edges(gpu):
    """freq_per_chan = polarizations = 2 with NaN-flagged entries, and
    measurements just inside u = 0, v = 0 and the far grid edges, whose
    support windows are clipped: the no-allocation binning and scatter run
    with their own parameters (no sub-counters, no partial tiles), so they are
    checked here against wstack() at 1e-12."""
    import torch

    import lofar_gb300 as L
    from lofar_gb300 import _lib

    lib = _lib.load()
    L.set_precision("fp64")
    rng = np.random.default_rng(31)
    nx, ny, planes, support, nf, npol = 96, 80, 4, 7, 2, 2
    n = 20_000
    uu = rng.random(n)
    vv = rng.random(n)
    edge = rng.choice(n, 4000, replace=False)
    side = rng.integers(0, 4, edge.size)
    eps = rng.random(edge.size) * 2.5 / nx
    uu[edge[side == 0]] = eps[side == 0]                          # just inside u = 0
    vv[edge[side == 1]] = eps[side == 1]                          # just inside v = 0
    uu[edge[side == 2]] = np.minimum(1.0 - eps[side == 2], np.nextafter(1.0, 0.0))
    vv[edge[side == 3]] = np.minimum(1.0 - eps[side == 3], np.nextafter(1.0, 0.0))
    ww = rng.random(n) * 0.999
    vr = rng.standard_normal(n * nf * npol).astype(np.float32)
    vi = rng.standard_normal(n * nf * npol).astype(np.float32)
    vr[rng.choice(vr.size, 500, replace=False)] = np.nan           # flagged: skipped
    wt = rng.random(n * npol).astype(np.float32)
    ref = np.zeros((planes, ny, nx, 2))
    L.wstack(planes, n, nf, npol, uu, vv, ww, vr, vi, wt, 1.0 / nx, 1.0 / planes, support, nx,
             ny, ref, 1)
    dev = [torch.as_tensor(a).cuda() for a in (uu, vv, ww, vr, vi, wt)]
    grid = torch.full((planes, ny, nx, 2), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        st = lib.wsg_grid_noalloc(planes, n, nf, npol, *(t.data_ptr() for t in dev), 1.0 / nx,
                                  1.0 / planes, support, nx, ny, grid.data_ptr(), None)
        assert st == _lib.WSG_OK, _lib.last_error()
        torch.cuda.synchronize()
        assert _nrm_max(grid.cpu().numpy(), ref) <= 1e-12
