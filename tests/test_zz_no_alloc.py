"""qmc_wf_psi_static: the psi entry point for callers that cannot allocate
device memory on the call path (an application that gives its whole HBM
budget to its own pool allocator, a latency-critical loop that must not let
cudaMalloc/cudaFree synchronize the device, a foreign-language binding with no
allocator hook). Its workspace is a fixed array compiled into the library.

The wave function here is C6H6 cc-pVDZ with cas(2,2) determinants: each of
its explicit-mode determinants keeps per-walker LU copies of two 21 x 21
spin matrices (7 KB per walker), far beyond the 16 KB of shared memory a
block may give its determinant phase, so the kernel works in the static
array (in HBM) and not in shared memory. The GPU test calls it through the C
ABI twice in a row, with different batches, and checks both results against
the allocating entry point qmc_wf_psi on the same positions and against the
oracle's psi (FP64, 1e-10 and 1e-9 relative). This file is collected last on
purpose."""
import ctypes

import numpy as np
import pytest
import torch

from qmctorch_gb300 import _lib
from tests.golden_cases import load

QMC_ERR_STATIC_LIMIT = 6
STATIC_BYTES = 16 * 1024 * 1024
SMEM_DET_BYTES = 16384  # largest determinant workspace a block keeps in shared memory
MIN_WALKERS_PER_BLOCK = 8


def _wavefunction():
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    mol, d = load("c6h6")
    wf = SlaterJastrow(mol, configs="cas(2,2)", include_all_mo=True, cuda=True)
    g = torch.Generator().manual_seed(5)
    wf.fc.weight.data = torch.rand(wf.fc.weight.shape, generator=g).cuda()
    return mol, d, wf


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.gpu
def test_static_scratch_psi_matches_allocating_entry_point_and_oracle():
    from oracle import qmc_oracle as orc
    mol, d, wf = _wavefunction()
    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    call = wf._desc(dev)
    per_walker = lib.qmc_scratch_bytes(call.ref, 32, 0) // 32
    assert per_walker * MIN_WALKERS_PER_BLOCK > SMEM_DET_BYTES  # the static array is used
    ow = orc.OracleSlaterJastrow(mol, configs="cas(2,2)", include_all_mo=True,
                                 fc_weight=wf.fc.weight.detach().cpu().numpy().reshape(-1))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(2024)
    for nw in (300, 77):  # two calls in a row, the second smaller than the first
        base = d["pos"][rng.integers(0, len(d["pos"]), nw)]
        pos_np = base + 0.3 * rng.normal(size=base.shape)
        pos = torch.as_tensor(pos_np, device=dev)
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
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, ref.cpu().numpy(), rtol=1e-10, atol=0)
        np.testing.assert_allclose(got, ow.forward(pos_np).ravel(), rtol=1e-9, atol=0)


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
