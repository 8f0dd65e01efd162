"""The asynchronous host calls (wsg_image_forward_host_async,
wsg_image_adjoint_host_async, wsg_plan_synchronize) against the blocking ones.

A stream of steps alternates two observations of different sizes, so the two
input slots, the image round trip through host memory and the output buffers
are all reused while earlier steps are still in flight.  Each step's outputs
must equal the blocking calls' outputs for the same observation (relative
max error 1e-6: the same kernels run in the same order).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, PLANES, SUPPORT = 512, 8, 7


def _obs(n, seed):
    from lofar_gb300 import synth
    o = synth.observe(n_stations=30, diameter_m=3000.0, hours=4.0, n_vis=n, sky_seed=seed,
                      noise_seed=seed + 1)
    return o


def _pinned(o):
    import torch
    return [torch.as_tensor(np.ascontiguousarray(getattr(o, k))).pin_memory()
            for k in ("uu", "vv", "ww", "vis_real", "vis_img", "weight")]


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def test_async_stream_matches_blocking_calls(gpu):
    import torch
    from lofar_gb300 import Plan
    obs = [_obs(200_000, 2), _obs(130_000, 7)]
    ins = [_pinned(o) for o in obs]
    plan = Plan(NX, NX, PLANES, SUPPORT, precision="fp32c")
    o0 = obs[0]
    plan.set_wcorrection(o0.resolution, o0.wmin, o0.wmax)
    ref = []
    for k, a in enumerate(ins):
        img = torch.empty((NX, NX), dtype=torch.complex64).pin_memory()
        vis = torch.empty(a[0].numel(), dtype=torch.complex64).pin_memory()
        plan.image_forward_host(*a, img)
        plan.image_adjoint_host(img, vis)
        ref.append((img.numpy().copy(), vis.numpy().copy()))
    steps = [0, 1, 0, 1, 1, 0]
    outs = []
    for k in steps:
        a = ins[k]
        img = torch.empty((NX, NX), dtype=torch.complex64).pin_memory()
        vis = torch.empty(a[0].numel(), dtype=torch.complex64).pin_memory()
        plan.image_forward_host_async(*a, img)
        plan.image_adjoint_host_async(img, vis)
        outs.append((k, img, vis))
    plan.synchronize()
    for k, img, vis in outs:
        assert _rel(img.numpy(), ref[k][0]) <= 1e-6
        assert _rel(vis.numpy(), ref[k][1]) <= 1e-6
    plan.close()


def test_async_adjoint_of_a_given_image(gpu):
    """The adjoint's image need not come from the forward call."""
    import torch
    from lofar_gb300 import Plan
    o = _obs(100_000, 4)
    a = _pinned(o)
    plan = Plan(NX, NX, PLANES, SUPPORT, precision="fp32c")
    plan.set_wcorrection(o.resolution, o.wmin, o.wmax)
    img = torch.empty((NX, NX), dtype=torch.complex64).pin_memory()
    g = torch.Generator().manual_seed(1)
    given = torch.randn((NX, NX), dtype=torch.complex64, generator=g).pin_memory()
    vis_ref = torch.empty(a[0].numel(), dtype=torch.complex64).pin_memory()
    plan.image_forward_host(*a, img)
    plan.image_adjoint_host(given, vis_ref)
    vis = torch.empty_like(vis_ref).pin_memory()
    plan.image_forward_host_async(*a, img)
    plan.image_adjoint_host_async(given, vis)
    plan.synchronize()
    assert _rel(vis.numpy(), vis_ref.numpy()) <= 1e-6
    plan.close()
