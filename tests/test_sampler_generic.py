"""Walker initialisation and Metropolis sampling of an arbitrary density,
against outputs of the reference itself (``tests/golden/walkers.npz`` and
``tests/golden/metropolis_generic.npz``, written by
``tests/golden/make_golden.py``).

Both are host code that must make the reference's random draws in the
reference's order (walkers.py:41-150; metropolis.py:85-298), so the bar is
equality to 1e-13 (the positions are sums of the same FP64 draws)."""
import os

import numpy as np
import pytest
import torch

from tests.golden_cases import GOLDEN

WALKER_CASES = ("h2o_sd", "lih_cas")
WALKER_METHODS = ("atomic", "center", "uniform", "normal")
WALKER_SEEDS = (31, 32)
WALKER_NW = 40

MGEN = {"nwalkers": 16, "nelec": 2, "ndim": 3, "nstep": 24, "step_size": 0.4,
        "ntherm": -8, "ndecor": 2, "seed": 4040}
MGEN_CASES = (("all-elec", "normal", False), ("one-elec", "uniform", False),
              ("all-elec-iter", "normal", False), ("all-elec", "normal", True),
              ("one-elec", "normal", False), ("all-elec-iter", "uniform", True))


def _gold(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        return {k: f[k] for k in f.files}


def _density():
    # the analytic density of the fixture: exp(-sum_k a_k (x_k - c_k)^2)
    rng = np.random.default_rng(5)
    a = torch.as_tensor(rng.uniform(0.4, 1.6, size=6))
    c = torch.as_tensor(rng.uniform(-0.5, 0.5, size=6))

    def pdf(x):
        return torch.exp(-(a.to(x.device) * (x - c.to(x.device)) ** 2).sum(-1))
    return pdf, a, c


@pytest.mark.parametrize("case", WALKER_CASES)
@pytest.mark.parametrize("method", WALKER_METHODS)
def test_walker_initialisation_matches_reference(case, method):
    from qmctorch_gb300.sampler.metropolis import Walkers
    from tests.golden_cases import load
    torch.set_default_dtype(torch.float64)
    mol, _ = load(case)
    ref = _gold("walkers")["%s_%s" % (case, method)]
    torch.manual_seed(WALKER_SEEDS[0])
    np.random.seed(WALKER_SEEDS[1])
    w = Walkers(nwalkers=WALKER_NW, nelec=mol.nelec, ndim=3, init=mol.domain(method))
    w.initialize()
    np.testing.assert_allclose(w.pos.numpy(), ref, rtol=0, atol=1e-13)


@pytest.mark.parametrize("icase", range(len(MGEN_CASES)))
def test_metropolis_on_arbitrary_density_matches_reference(icase):
    from qmctorch_gb300.sampler import Metropolis
    torch.set_default_dtype(torch.float64)
    gold = _gold("metropolis_generic")
    pdf, _, _ = _density()
    mtype, proba, logspace = MGEN_CASES[icase]
    g = MGEN
    sampler = Metropolis(nwalkers=g["nwalkers"], nstep=g["nstep"], step_size=g["step_size"],
                         ntherm=g["ntherm"], ndecor=g["ndecor"], nelec=g["nelec"], ndim=g["ndim"],
                         init={"method": "uniform", "min": -1, "max": 1},
                         move={"type": mtype, "proba": proba}, logspace=logspace)
    torch.manual_seed(g["seed"] + icase)
    samples = sampler(pdf, pos=torch.as_tensor(gold["pos0"]).clone(), with_tqdm=False)
    np.testing.assert_allclose(samples.detach().numpy(), gold["samples_%d" % icase],
                               rtol=0, atol=1e-13)
    np.testing.assert_allclose(sampler.walkers.pos.numpy(), gold["final_%d" % icase],
                               rtol=0, atol=1e-13)


def test_metropolis_construction_draws_nothing():
    """Building a sampler leaves torch's generator alone (the reference's
    constructor draws nothing), so a seed set before construction gives the
    reference's chain."""
    from qmctorch_gb300.sampler import Metropolis
    torch.manual_seed(5)
    a = torch.rand(3)
    torch.manual_seed(5)
    Metropolis(nwalkers=4, nstep=2, nelec=2, init={"method": "uniform", "min": -1, "max": 1})
    np.testing.assert_array_equal(torch.rand(3).numpy(), a.numpy())


def test_replay_needs_a_wave_function():
    from qmctorch_gb300.sampler import Metropolis
    pdf, _, _ = _density()
    s = Metropolis(nwalkers=4, nstep=2, nelec=2, init={"method": "uniform", "min": -1, "max": 1})
    with pytest.raises(ValueError):
        s(pdf, pos=torch.zeros(4, 6, dtype=torch.float64), replay={"proposals": None})


HMC = {"nwalkers": 16, "nelec": 2, "ndim": 3, "nstep": 12, "step_size": 0.1, "L": 6,
       "ntherm": -6, "ndecor": 2, "seed": 777}


def _hmc():
    from qmctorch_gb300.sampler import Hamiltonian
    g = HMC
    return Hamiltonian(nwalkers=g["nwalkers"], nstep=g["nstep"], step_size=g["step_size"],
                       L=g["L"], ntherm=g["ntherm"], ndecor=g["ndecor"], nelec=g["nelec"],
                       ndim=g["ndim"], init={"method": "uniform", "min": -1, "max": 1})


def test_hamiltonian_on_arbitrary_density_matches_reference():
    """HMC (hamiltonian.py:10-201) with autograd forces on the analytic
    density: the reference's chain to 1e-13."""
    torch.set_default_dtype(torch.float64)
    gold = _gold("hamiltonian")
    pdf, _, _ = _density()
    s = _hmc()
    torch.manual_seed(HMC["seed"])
    samples = s(pdf, pos=torch.as_tensor(gold["pos0"]), with_tqdm=False)
    np.testing.assert_allclose(samples.detach().numpy(), gold["samples"], rtol=0, atol=1e-13)
