"""The block-cooperative LU of the psi / Metropolis determinant phase (spin
channels of six or more electrons beyond the register path: the threads of a
walker share the elimination steps).

* psi and E_L of H12, H20 and H24 sto-3g chains (ground state, n = 6, 10
  and 12 per spin) against the FP64 oracle within the rounding bound of each
  walker's Slater matrices (condition numbers up to 1e10 at these positions);
  the mixed method within 1e-3 relative (median) at H12, where FP32 MO values
  allow it (kappa ~ 1e5; the longer chains are beyond the mixed method);
* psi is bitwise the same whatever the launch plan's threads per walker
  (16384 walkers vs. a 37-walker subset);
* the local-energy kernel (its own cooperative factorisation of copies of
  the same rows, cooperative column solves) gives the oracle's local energy
  and the psi kernel's psi within that bound (mixed at H12: 1e-2 Ha median);
* an FP64 Metropolis chain of H20 replays the oracle's chain.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import qmc_oracle as orc

pytestmark = pytest.mark.gpu


def _mol(n):
    from qmctorch_gb300.scf import Molecule
    from qmctorch_gb300.serving import hydrogen_chain
    return Molecule(hydrogen_chain(n, 0.95), unit="angs", basis="sto-3g", calculator="huckel")


def _wf(mol, precision):
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    return SlaterJastrow(mol, cuda=True, precision=precision)


def _psi_from_local_energy(wf, x):
    from qmctorch_gb300 import _lib
    from qmctorch_gb300.wavefunction import runtime as rt
    lib = _lib.lib()
    call = wf._desc(x.device)
    nb = x.shape[0]
    scr = rt.scratch(lib.qmc_scratch_bytes(call.ref, nb, 1), x.device)
    el = torch.empty(nb, dtype=torch.float64, device=x.device)
    psi = torch.empty(nb, dtype=torch.float64, device=x.device)
    _lib.check(lib.qmc_wf_local_energy(call.ref, rt.ptr(x), nb, rt.ptr(el), None, rt.ptr(psi),
                                       rt.ptr(scr), scr.numel(), rt.stream_handle()),
               "qmc_wf_local_energy")
    return psi


def _rtol_from_conditioning(ow, pos):
    """Per-walker bound on the relative rounding error of an FP64 psi: the
    Slater matrices of these chains at sampled positions have condition
    numbers up to 1e10, and a backward-stable LU's determinant is accurate to
    about n eps kappa (either implementation, summation orders differ)."""
    from oracle.qmc_oracle import ao_values
    mo = ao_values(ow.basis, pos, 0) @ ow.W
    nu = ow.nup
    k = np.array([np.linalg.cond(m[:nu, :nu]) + np.linalg.cond(m[nu:, :ow.ndown]) for m in mo])
    return 1e-12 + 1e-16 * 8 * nu * k


@pytest.mark.parametrize("n", [12, 20, 24])
def test_psi_against_oracle_and_plans(n):
    from qmctorch_gb300.serving import seeded_positions
    mol = _mol(n)
    wf64, wfm = _wf(mol, "fp64"), _wf(mol, "mixed")
    big = torch.as_tensor(seeded_positions(mol, 16384, seed=n), device="cuda")
    ow = orc.OracleSlaterJastrow(mol, configs="ground_state", include_all_mo=True,
                                 fc_weight=np.ones(1))
    pos = big[:8].cpu().numpy()
    with torch.no_grad():
        p64 = wf64(big)
        pm = wfm(big)
        got = p64[:8].cpu().numpy().ravel()
        ref = ow.forward(pos).ravel()
        assert np.all(np.abs(got - ref) <= _rtol_from_conditioning(ow, pos) * np.abs(ref))
        rel = ((pm - p64) / p64).abs()
        # FP32 MO values limit the mixed method to about kappa * 6e-8 relative:
        # median 2.5e-4 at H12 (kappa ~ 1e5), of order 1 at H20 (kappa ~ 1e9)
        if n == 12:
            assert float(rel.median()) < 1e-3, float(rel.median())
        for wf, full in ((wf64, p64), (wfm, pm)):
            np.testing.assert_array_equal(wf(big[:37].clone()).cpu().numpy(),
                                          full[:37].cpu().numpy())
        el = wf64.local_energy(big[:8].clone()).cpu().numpy().ravel()
        el_ref = ow.local_energy(pos).ravel()
        assert np.all(np.abs(el - el_ref) <= _rtol_from_conditioning(ow, pos) * (np.abs(el_ref) + 1))
        if n == 12:
            elm = wfm.local_energy(big[:64].clone()).cpu().numpy().ravel()
            el64 = wf64.local_energy(big[:64].clone()).cpu().numpy().ravel()
            assert np.median(np.abs(elm - el64)) < 1e-2
        q = _psi_from_local_energy(wf64, big[:512].contiguous()).cpu().numpy()
        ref = p64[:512].cpu().numpy().ravel()
        tol = _rtol_from_conditioning(ow, big[:512].cpu().numpy())
        assert np.all(np.abs(q - ref) <= tol * np.abs(ref))


def test_metropolis_replay_h20():
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.serving import seeded_positions
    mol = _mol(20)
    wf = _wf(mol, "fp64")
    ow = orc.OracleSlaterJastrow(mol, configs="ground_state", include_all_mo=True,
                                 fc_weight=np.ones(1))
    nw, nstep = 8, 6
    rng = np.random.default_rng(5)
    pos0 = seeded_positions(mol, nw, seed=7)
    props = rng.normal(size=(nstep, nw, 3 * mol.nelec)) * orc.metropolis_sigma(0.2)
    unif = rng.uniform(size=(nstep, nw))
    ref, _, _ = orc.metropolis_replay(ow.pdf, pos0, props, unif, ntherm=0, ndecor=1)
    s = Metropolis(nwalkers=nw, nstep=nstep, step_size=0.2, ntherm=0, ndecor=1, nelec=mol.nelec,
                   init=mol.domain("atomic"), cuda=True)
    out = s(wf.pdf, pos=torch.as_tensor(pos0, device="cuda"), with_tqdm=False,
            replay={"proposals": props, "uniforms": unif})
    np.testing.assert_allclose(out.detach().cpu().numpy(), np.asarray(ref).reshape(out.shape),
                               rtol=0, atol=1e-12)
