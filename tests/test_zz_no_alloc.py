"""qmc_wf_psi_static: the psi entry point for callers that cannot allocate
device memory on the call path (an application that gives its whole HBM
budget to its own pool allocator, a latency-critical loop that must not let
cudaMalloc/cudaFree synchronize the device, a foreign-language binding with no
allocator hook). Its workspace is a fixed array compiled into the library.

The GPU test calls it through the C ABI twice in a row, with different
batches, and checks both results against the allocating entry point
qmc_wf_psi on the same positions (FP64, 1e-10 relative: the same kernel runs
on the same inputs). This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from qmctorch_gb300 import _lib
from tests.golden_cases import load

QMC_ERR_STATIC_LIMIT = 6
STATIC_BYTES = 16 * 1024 * 1024


def _wavefunction():
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    mol, d = load("h2o_sd")
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"], cuda=True)
    wf.fc.weight.data = torch.as_tensor(d["fc_weight"], device="cuda").reshape(1, -1)
    return mol, d, wf


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.gpu
def test_static_scratch_psi_matches_allocating_entry_point():
    mol, d, wf = _wavefunction()
    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    call = wf._desc(dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(2024)
    for nw in (1000, 77):  # two calls in a row, the second smaller than the first
        base = d["pos"][rng.integers(0, len(d["pos"]), nw)]
        pos = torch.as_tensor(base + 0.4 * rng.normal(size=base.shape), device=dev)
        need = lib.qmc_scratch_bytes(call.ref, nw, 0)
        assert 0 < need <= STATIC_BYTES
        scr = torch.empty(need, dtype=torch.uint8, device=dev)
        ref = torch.empty(nw, dtype=torch.float64, device=dev)
        st = lib.qmc_wf_psi(call.ref, _p(pos), nw, _p(ref), _p(scr), need, stream)
        assert st == 0
        out = torch.full((nw,), float("nan"), dtype=torch.float64, device=dev)
        st = lib.qmc_wf_psi_static(call.ref, _p(pos), nw, _p(out), stream)
        assert st == 0, lib.qmc_status_string(st)
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), ref.cpu().numpy(), rtol=1e-10, atol=0)


@pytest.mark.gpu
def test_static_scratch_psi_rejects_oversized_batch():
    mol, d, wf = _wavefunction()
    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    call = wf._desc(dev)
    per_walker = lib.qmc_scratch_bytes(call.ref, 32, 0) // 32
    too_many = STATIC_BYTES // per_walker + 64
    dummy = torch.zeros(3 * mol.nelec, dtype=torch.float64, device=dev)
    st = lib.qmc_wf_psi_static(call.ref, _p(dummy), too_many, _p(dummy), None)
    assert st == QMC_ERR_STATIC_LIMIT
    assert b"static" in lib.qmc_status_string(st)
