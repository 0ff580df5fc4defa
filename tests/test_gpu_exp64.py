"""GPU test of the FP64 exponential the fused kernels use for their radial
factors (Tang's table-driven method, qmc_device.cuh exp_tang) against the
library exp (torch.exp on the GPU): within 2 units in the last place over the
radial arguments [-707, 0] (dense near 0, where the dominant primitives sit,
and uniform across the range), over positive arguments up to 707, at the
table's boundaries (multiples of ln2 / 64 and the half-way points), and the
library's own values outside the fast range (subnormal results, overflow,
infinities, NaN)."""
import ctypes
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def kernel_exp(x):
    from qmctorch_gb300 import _lib
    lib = _lib.lib()
    xd = torch.as_tensor(x, dtype=torch.float64, device="cuda").contiguous()
    y = torch.empty_like(xd)
    st = lib.qmc_probe_exp64(ctypes.c_void_p(xd.data_ptr()), xd.numel(),
                             ctypes.c_void_p(y.data_ptr()),
                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    return xd, y


def ulps(y, ref):
    spacing = np.spacing(np.abs(ref))
    return np.abs(y - ref) / spacing


def test_exp_tang_within_two_ulp():
    rng = np.random.default_rng(3)
    c = math.log(2.0) / 64
    xs = np.concatenate([
        -np.abs(rng.standard_normal(200_000)) * 2.0,       # dominant primitives
        rng.uniform(-707.0, 0.0, 400_000),                  # the radial range
        rng.uniform(0.0, 707.0, 100_000),                   # positive arguments
        np.arange(-65000, 65000, 7) * c,                    # table boundaries
        (np.arange(-65000, 65000, 7) + 0.5) * c,            # half-way points
        np.array([0.0, -0.0, 1e-300, -1e-300, 1e-10, -1e-10, -706.99, 706.99]),
    ])
    x, y = kernel_exp(xs)
    ref = torch.exp(x).cpu().numpy()
    y = y.cpu().numpy()
    u = ulps(y, ref)
    assert float(u.max()) <= 2.0, (float(u.max()), float(xs[np.argmax(u)]))
    assert float(u.mean()) < 0.5


def test_exp_tang_outside_the_fast_range_is_the_library_exp():
    xs = np.array([-707.0, -720.0, -745.0, -746.0, -1e4, 707.5, 709.7, 710.0, np.inf, -np.inf,
                   np.nan])
    x, y = kernel_exp(xs)
    ref = torch.exp(x).cpu().numpy()
    y = y.cpu().numpy()
    np.testing.assert_array_equal(np.isnan(y), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.array_equal(y[ok], ref[ok])
