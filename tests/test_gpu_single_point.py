"""``Solver.single_point`` on the H2 configuration (solver_base.py:316-387,
wf_base.py:225-229): H2 at +-0.37 A, sto-3g, one determinant with the Pade
e-e Jastrow, 4096 walkers, all-electron Gaussian moves of step 0.2, 500
steps of which 200 are burn-in, every later step kept (1,228,800 samples).

* the returned statistics are those of the returned local energies:
  ``energy`` = their mean, ``variance`` = ``torch.var`` (unbiased),
  ``error`` = sqrt(variance / n), each to 1e-12 relative;
* the energy agrees within 3 sigma with the oracle's sampled energy (the
  oracle's Metropolis chain on the CPU with independent random numbers),
  sigma from the spread of per-walker mean energies of both runs (walkers are
  independent chains, snapshots of one walker are not).
"""
import numpy as np
import pytest
import torch

from oracle import qmc_oracle as orc
from tests.golden_cases import load

pytestmark = pytest.mark.gpu

NW, NSTEP, NTHERM, STEP = 4096, 500, 200, 0.2


def walker_means(eloc, nsnap, nw):
    m = np.asarray(eloc).reshape(nsnap, nw).mean(0)
    return m.mean(), m.std(ddof=1) / np.sqrt(nw)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_single_point_h2(precision):
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.solver import Solver
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    mol, _ = load("h2")
    wf = SlaterJastrow(mol, configs="ground_state", cuda=True, precision=precision)
    sampler = Metropolis(nwalkers=NW, nstep=NSTEP, step_size=STEP, ntherm=NTHERM, ndecor=1,
                         nelec=mol.nelec, init=mol.domain("atomic"), cuda=True, seed=77)
    solver = Solver(wf=wf, sampler=sampler)
    torch.manual_seed(0)
    np.random.seed(0)
    obs = solver.single_point(with_tqdm=False)
    nsnap = NSTEP - NTHERM
    assert obs.pos.shape == (nsnap * NW, 3 * mol.nelec)
    el = obs.local_energy.detach().reshape(-1)
    assert el.numel() == nsnap * NW
    n = el.numel()
    var = torch.var(el)
    assert abs(float(obs.energy) - float(el.mean())) <= 1e-12 * abs(float(el.mean()))
    assert abs(float(obs.variance) - float(var)) <= 1e-12 * float(var)
    assert abs(float(obs.error) - float(torch.sqrt(var / n))) <= 1e-12 * float(torch.sqrt(var / n))
    eg, sg = walker_means(el.cpu().numpy(), nsnap, NW)
    # oracle chain (CPU, numpy generator): 1024 walkers, 400 steps, every 10th kept
    ow = orc.OracleSlaterJastrow(mol, configs="ground_state")
    rng = np.random.default_rng(808)
    nwo, ostep, otherm, odecor = 1024, 400, 200, 10
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)
    pos0 = (centers[None] + rng.normal(size=(nwo, mol.nelec, 3))).reshape(nwo, -1)
    props = rng.normal(size=(ostep, nwo, 3 * mol.nelec)) * orc.metropolis_sigma(STEP)
    unif = rng.uniform(size=(ostep, nwo))
    samples, _, _ = orc.metropolis_replay(ow.pdf, pos0, props, unif, ntherm=otherm, ndecor=odecor)
    eo, so = walker_means(ow.local_energy(samples), len(range(otherm, ostep, odecor)), nwo)
    assert abs(eg - eo) < 3 * np.sqrt(sg ** 2 + so ** 2), (eg, eo, sg, so)
    assert abs(float(obs.energy) - eg) < 1e-12
