"""GPU tests of the drift-diffusion sampler on wave functions of this package
(one qmc_drift_run launch per call).

* With ``rng="torch"`` the kernel consumes the reference's random draws, so
  its chains are compared with the chains of the reference's
  GeneralizedMetropolis on its own H2 sto-3g SlaterJastrow (autograd drift),
  same seed and initial walkers (tests/golden/gmetropolis.npz). Tolerance:
  1e-9 absolute on the positions (FP64 density and drift agree with the
  reference's to about 1e-14; the accept / reject decisions are the same).
* On H2O cc-pVDZ single_double(4,4), LiH cas(2,2), their electron-nucleus and
  combined Jastrow cases and LiH with Slater-type orbitals the kernel is compared
  with this package's host loop (density by qmc_wf_psi, drift by
  qmc_wf_gradients) on the same draws: same tolerance.
* With the device generator the chains are reproducible, keep the proposal
  rule (a kept position differs from the call's start positions in at most
  one electron), and accept at the rate of the torch-drawn chains.
"""
import os

import numpy as np
import pytest
import torch

from tests.golden_cases import load
from tests.golden_cases import make_wf as golden_make_wf

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gmetropolis.npz")


def make_wf(name):
    """The case's wave function (its Jastrow factors: e-e, e-n or both; GTO or STO)."""
    mol, d = load(name)
    return mol, d, golden_make_wf(mol, d)


class HostLoopPdf:
    """wf.pdf under another name: the sampler runs its host loop, with the
    drift from the wave function's Jacobi gradient kernel."""

    def __init__(self, wf):
        self.__self__ = wf
        self.__name__ = "pdf_host_loop"

    def __call__(self, x, return_grad=False):
        return self.__self__.pdf(x, return_grad=return_grad)


def test_drift_sampler_chains_match_the_reference_on_h2():
    from qmctorch_gb300.sampler import GeneralizedMetropolis
    from qmctorch_gb300.wavefunction import SlaterJastrow
    with np.load(GOLDEN) as f:
        g = {k: f[k] for k in f.files}
    torch.set_default_dtype(torch.float64)
    mol, d = load("h2")
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"], cuda=True)
    s = GeneralizedMetropolis(nwalkers=16, nstep=20, step_size=0.2, ntherm=-10, ndecor=2,
                              nelec=mol.nelec, ndim=3, cuda=True, rng="torch",
                              init={"method": "uniform", "min": -1, "max": 1})
    torch.manual_seed(int(g["cfg_seed"]) + 1)
    out = s(wf.pdf, pos=torch.as_tensor(g["h2_pos0"], device="cuda"), with_tqdm=False)
    assert out.is_cuda and out.shape == g["h2_samples"].shape
    np.testing.assert_allclose(out.detach().cpu().numpy(), g["h2_samples"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(s.walkers.pos.cpu().numpy(), g["h2_final"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("name", ["h2o_sd", "lih_cas", "h2o_en", "lih_en", "lih_sto"])
def test_drift_kernel_matches_the_host_loop(name):
    from qmctorch_gb300.sampler import GeneralizedMetropolis
    mol, d, wf = make_wf(name)
    nw = 512
    rng = np.random.default_rng(7)
    pos0 = torch.as_tensor(np.repeat(d["pos"], -(-nw // len(d["pos"])), axis=0)[:nw]
                           + 0.05 * rng.standard_normal((nw, 3 * mol.nelec)), device="cuda")
    runs = []
    for pdf in (wf.pdf, HostLoopPdf(wf)):
        s = GeneralizedMetropolis(nwalkers=nw, nstep=40, step_size=0.05, ntherm=-20, ndecor=3,
                                  nelec=mol.nelec, ndim=3, cuda=True, rng="torch")
        torch.manual_seed(1234)
        out = s(pdf, pos=pos0.clone(), with_tqdm=False)
        runs.append((out.detach().cpu().numpy(), s.walkers.pos.cpu().numpy()))
    (ko, kf), (ho, hf) = runs
    assert ko.shape == ho.shape == (7 * nw, 3 * mol.nelec)
    moved = np.abs(ko - np.tile(pos0.cpu().numpy(), (7, 1))).max(axis=1) > 0
    assert moved.mean() > 0.2  # the chains do move
    np.testing.assert_allclose(ko, ho, rtol=0, atol=1e-9)
    np.testing.assert_allclose(kf, hf, rtol=0, atol=1e-9)


def test_device_generator_chains():
    from qmctorch_gb300.sampler import GeneralizedMetropolis
    mol, d, wf = make_wf("h2o_sd")
    nw, nstep = 4096, 30
    rng = np.random.default_rng(11)
    pos0 = torch.as_tensor(np.repeat(d["pos"], -(-nw // len(d["pos"])), axis=0)[:nw]
                           + 0.05 * rng.standard_normal((nw, 3 * mol.nelec)), device="cuda")

    def run(kind, seed):
        s = GeneralizedMetropolis(nwalkers=nw, nstep=nstep, step_size=0.05, ntherm=0, ndecor=1,
                                  nelec=mol.nelec, ndim=3, cuda=True, rng=kind, seed=seed)
        torch.manual_seed(99)
        out = s(wf.pdf, pos=pos0.clone(), with_tqdm=False)
        return out.detach().cpu().numpy(), s.last_acceptance

    a, acc_a = run("device", 5)
    b, acc_b = run("device", 5)
    c, acc_c = run("device", 6)
    t, acc_t = run("torch", None)
    assert np.array_equal(a, b) and acc_a == acc_b
    assert not np.array_equal(a, c)
    # proposals start from the call's start positions: one electron moved at most
    dif = np.abs(a - np.tile(pos0.cpu().numpy(), (nstep, 1))).reshape(nstep * nw, mol.nelec, 3)
    assert (dif.max(axis=2) > 0).sum(axis=1).max() == 1
    moved_e = np.argmax(dif.max(axis=2), axis=1)[dif.max(axis=(1, 2)) > 0]
    counts = np.bincount(moved_e, minlength=mol.nelec)
    assert counts.min() > 0.5 * counts.mean()  # every electron is drawn
    assert 0.05 < acc_t < 0.95
    assert abs(acc_a - acc_t) < 0.02 and abs(acc_c - acc_t) < 0.02
