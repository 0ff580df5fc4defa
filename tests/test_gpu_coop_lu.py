"""The block-cooperative LU of the psi / Metropolis determinant phase (spin
channels of six or more electrons beyond the register path: the threads of a
walker share the elimination steps).

* psi of H20 and H24 sto-3g chains (ground state, n = 10 and 12 per spin)
  against the FP64 oracle (1e-10 relative), the mixed method within 1e-5 relative (median);
* psi is bitwise the same whatever the launch plan's threads per walker
  (16384 walkers vs. a 37-walker subset);
* the local-energy kernel, which factors with one thread per channel, gives
  the same psi (FP64: the same operations; 1e-13 relative);
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


@pytest.mark.parametrize("n", [20, 24])
def test_psi_against_oracle_and_plans(n):
    from qmctorch_gb300.serving import seeded_positions
    mol = _mol(n)
    wf64, wfm = _wf(mol, "fp64"), _wf(mol, "mixed")
    big = torch.as_tensor(seeded_positions(mol, 16384, seed=n), device="cuda")
    ow = orc.OracleSlaterJastrow(mol, configs="ground_state", include_all_mo=True,
                                 fc_weight=np.ones(1))
    pos = big[:6].cpu().numpy()
    with torch.no_grad():
        p64 = wf64(big)
        pm = wfm(big)
        np.testing.assert_allclose(p64[:6].cpu().numpy().ravel(), ow.forward(pos).ravel(),
                                   rtol=1e-10, atol=0)
        rel = ((pm - p64) / p64).abs()
        # the mixed method's per-walker error grows near the nodes of psi
        assert float(rel.median()) < 1e-5 and float(rel.quantile(0.99)) < 1e-3
        for wf, full in ((wf64, p64), (wfm, pm)):
            np.testing.assert_array_equal(wf(big[:37].clone()).cpu().numpy(),
                                          full[:37].cpu().numpy())
        q = _psi_from_local_energy(wf64, big[:512].contiguous())
        np.testing.assert_allclose(q.cpu().numpy(), p64[:512].cpu().numpy().ravel(), rtol=1e-13,
                                   atol=0)


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
