"""Statistical agreement of sampled VMC energies: the GPU sampler (plain FP64
and mixed methods) against the oracle's Metropolis chain on the CPU, run
with independent random numbers. The energies must agree within 3 sigma,
sigma from the spread of per-walker mean energies (walkers are independent
chains)."""
import numpy as np
import pytest
import torch

from oracle import qmc_oracle as orc
from tests.golden_cases import load

pytestmark = pytest.mark.gpu


def walker_means(eloc, nsnap, nw):
    e = np.asarray(eloc).reshape(nsnap, nw)
    m = e.mean(0)
    return m.mean(), m.std(ddof=1) / np.sqrt(nw)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sampled_energy_agrees_with_oracle_h2(precision):
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    mol, d = load("h2")
    step, nstep, ntherm, ndecor = 0.2, 400, 200, 10
    nsnap = len(range(ntherm, nstep, ndecor))
    # oracle chain (CPU, numpy generator)
    ow = orc.OracleSlaterJastrow(mol, configs="ground_state")
    rng = np.random.default_rng(2024)
    nwo = 1024
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)
    pos0 = (centers[None] + rng.normal(size=(nwo, 2, 3))).reshape(nwo, -1)
    props = rng.normal(size=(nstep, nwo, 6)) * orc.metropolis_sigma(step)
    unif = rng.uniform(size=(nstep, nwo))
    samples, _, _ = orc.metropolis_replay(ow.pdf, pos0, props, unif, ntherm=ntherm, ndecor=ndecor)
    eo, so = walker_means(ow.local_energy(samples), nsnap, nwo)
    # GPU chain (Philox generator)
    wf = SlaterJastrow(mol, configs="ground_state", cuda=True, precision=precision)
    nwg = 8192
    x0 = torch.as_tensor((centers[None] + rng.normal(size=(nwg, 2, 3))).reshape(nwg, -1),
                         device="cuda")
    sampler = Metropolis(nwalkers=nwg, nstep=nstep, step_size=step, ntherm=ntherm, ndecor=ndecor,
                         nelec=2, init=mol.domain("atomic"), cuda=True, seed=99)
    pos = sampler(wf.pdf, pos=x0, with_tqdm=False)
    eg, sg = walker_means(wf.local_energy(pos).detach().cpu().numpy(), nsnap, nwg)
    assert abs(eg - eo) < 3 * np.sqrt(so ** 2 + sg ** 2), (eg, eo, sg, so)
    assert sg < 5e-3 and so < 1e-2
