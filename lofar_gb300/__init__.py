"""GB300-native (sm_103a) w-stacking hot path of the HPC_Imaging/LOFAR imager.

The compute lives in ``libwstack_gb300.so`` (CUDA kernels behind a C ABI,
``include/wstack_gb300.h``); this package is its Python front end:

* ``api``       reference entry points (wstack, phase_correction, fft_planes)
                the device-resident ``Plan`` and the (channel, polarisation)
                ``Batch``
* ``autograd``  ``torch.autograd.Function`` over the forward imaging operator
                and its hand-written adjoint
* ``synth``     seeded synthetic observations in the reference's input layout
* ``binms``     the reference's parameter, meta and binary files, its dumps,
                and its main() as ``run``
* ``build``     the nvcc recipe that produces the shared library
"""
from ._lib import WSG_FP32C, WSG_FP64, WstackError  # noqa: F401
from .api import Batch, Plan, fft_planes, phase_correction, release, set_precision, wstack  # noqa: F401

__all__ = ["Plan", "Batch", "wstack", "phase_correction", "fft_planes", "set_precision", "release",
           "WstackError", "WSG_FP64", "WSG_FP32C"]
