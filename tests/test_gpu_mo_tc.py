"""GPU tests of the tensor-core AO->MO contraction (qmc_mo_eval_tc: tcgen05
MMAs, split-BF16 x3 operands, FP32 accumulators in tensor memory) against the
FP64 kernel (qmc_mo_eval) and the reference MO values of the golden fixtures.

Stated tolerance, elementwise: |MO_tc - MO_fp64| <= 5e-5 * (|AO| @ |W|)
(W = mo_scf * mo_modifier). The split keeps about 16 significant bits of each
operand, so the expected error is about 1.5e-5 of that bound; the factor
covers FP32 accumulation over up to 3 x 128 terms.
"""
import numpy as np
import pytest
import torch

from tests.golden_cases import load

pytestmark = pytest.mark.gpu

TOL = 5e-5


def make_wf(mol, d, precision):
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    return SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"],
                         cuda=True, precision=precision)


def seeded_positions(mol, nw, seed):
    rng = np.random.default_rng(seed)
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)[: mol.nelec]
    return torch.as_tensor((centers[None] + rng.normal(size=(nw, mol.nelec, 3))).reshape(nw, -1),
                           device="cuda")


def check_close(mo_tc, mo64, ao, wf):
    W = (wf.mo.mo_scf * wf.mo.mo_modifier).detach().to(torch.float64)
    bound = TOL * (ao.abs().reshape(-1, ao.shape[-1]) @ W.abs()).reshape(mo64.shape)
    err = (mo_tc - mo64).abs()
    assert torch.isfinite(mo_tc).all()
    assert bool((err <= bound + 1e-300).all()), float((err / (bound + 1e-300)).max())
    return float((err / (bound / TOL + 1e-300)).max())


# (case, walkers): rows = walkers x electrons cover a partial tile (h2: 6 rows),
# a ragged last tile, and more tiles than resident CTAs (persistent loop)
@pytest.mark.parametrize("name,nw", [("h2", 3), ("lih_cas", 333), ("h2o_sd", 1001),
                                     ("h2o_sd", 16384), ("c6h6", 97), ("c6h6", 4096)])
def test_tensor_core_mo_matches_fp64(name, nw):
    mol, d = load(name)
    wf64 = make_wf(mol, d, "fp64")
    wfmx = make_wf(mol, d, "mixed")
    assert wf64.mo.precision == "fp64" and wfmx.mo.precision == "mixed"
    x = seeded_positions(mol, nw, seed=nw)
    with torch.no_grad():
        ao = wf64.ao(x)
        mo64 = wf64.mo(ao)
        mo_tc = wfmx.mo(ao)
    assert mo_tc.shape == mo64.shape == (nw, mol.nelec, wf64.mo.mo_scf.shape[1])
    rel = check_close(mo_tc, mo64, ao, wf64)
    assert rel < 3e-5  # measured error relative to |AO| @ |W|, split-BF16 x3


@pytest.mark.parametrize("name", ["h2o_sd", "c6h6"])
def test_tensor_core_mo_against_reference_values(name):
    """On the golden positions: the reference's MO tensor (FP64 PyTorch)."""
    mol, d = load(name)
    wfmx = make_wf(mol, d, "mixed")
    with torch.no_grad():
        ao = torch.as_tensor(d["ao"], device="cuda") if "ao" in d else wfmx.ao(
            torch.as_tensor(d["pos"], device="cuda"))
        mo_tc = wfmx.mo(ao)
    ref = torch.as_tensor(d["mo"], device="cuda") if "mo" in d else make_wf(mol, d, "fp64").mo(ao)
    check_close(mo_tc, ref, ao, wfmx)


def test_tensor_core_mo_is_deterministic_and_follows_mo_modifier():
    mol, d = load("h2o_sd")
    wfmx = make_wf(mol, d, "mixed")
    wf64 = make_wf(mol, d, "fp64")
    x = seeded_positions(mol, 2048, seed=5)
    with torch.no_grad():
        ao = wf64.ao(x)
        a = wfmx.mo(ao)
        b = wfmx.mo(ao)
        assert torch.equal(a, b)
        g = torch.Generator().manual_seed(3)
        mod = 1.0 + 0.1 * torch.rand(wfmx.mo.mo_modifier.shape, generator=g)
        wfmx.mo.mo_modifier.data.copy_(mod.to(wfmx.mo.mo_modifier.device))
        wf64.mo.mo_modifier.data.copy_(mod.to(wf64.mo.mo_modifier.device))
        check_close(wfmx.mo(ao), wf64.mo(ao), ao, wf64)


def test_tensor_core_mo_reports_a_wait_that_ran_out():
    """With a pipeline wait limit of 0 every wait of the kernel gives up at
    once (nothing is waited for; no fault, no hang): the launch writes NaN
    rows, qmc_mo_eval_tc_status returns QMC_ERR_TIMEOUT and clears the status
    word, the module call raises, and with the default limit restored the
    next call is exact again."""
    from qmctorch_gb300 import _lib
    mol, d = load("h2o_sd")
    wfmx = make_wf(mol, d, "mixed")
    wf64 = make_wf(mol, d, "fp64")
    x = seeded_positions(mol, 4096, seed=11)
    lib = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    with torch.no_grad():
        ao = wf64.ao(x)
        mo64 = wf64.mo(ao)
        assert lib.qmc_mo_eval_tc_status(stream) == 0
        old = lib.qmc_set_wait_limit_ns(0)
        try:
            assert old == 1000000000
            with pytest.raises(_lib.QMCError, match="ran out"):
                wfmx.mo(ao)
            # the same launch through the C ABI: NaN rows and the status word
            from qmctorch_gb300.wavefunction import runtime as rt
            call = rt.build_desc(ao.device, wfmx.mo._ao_module, mo=wfmx.mo)
            a2 = ao.reshape(-1, ao.shape[-1]).contiguous()
            out = torch.zeros((a2.shape[0], mo64.shape[-1]), dtype=torch.float64,
                              device=ao.device)
            st = lib.qmc_mo_eval_tc(call.ref, a2.data_ptr(), a2.shape[0], out.data_ptr(), stream)
            assert st == 0
            assert lib.qmc_mo_eval_tc_status(stream) == 7
            assert bool(torch.isnan(out).all())
            assert lib.qmc_mo_eval_tc_status(stream) == 0  # cleared
        finally:
            lib.qmc_set_wait_limit_ns(old)
        check_close(wfmx.mo(ao), mo64, ao, wf64)
        assert lib.qmc_mo_eval_tc_status(stream) == 0
