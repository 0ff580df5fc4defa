"""Accept/reject parity at the headline configuration: H2O cc-pVDZ with
single_double(4,4) determinants and the Pade e-e Jastrow, 4096 walkers, 50
all-electron Gaussian moves of step 0.2 (metropolis.py:85-177, 279-298).

One set of proposals and uniforms is drawn once (seeded numpy) and replayed
into the oracle's sampler and into the GPU kernel.

Decision tolerance, the bar of this file:
* plain FP64 method: tau = 0 -- every one of the 4096 x 50 decisions equals
  the oracle's and the chains agree to 1e-12 bohr;
* mixed method: a decision may differ from the oracle's only where
  |min(1, r) - u| < TAU_MIXED = 1e-3 in the oracle's ratio r. The mixed
  method's psi is within 1e-4 relative of FP64 per walker, so r is within
  about 4e-4 relative and min(1, r) within 4e-4 absolute; 1e-3 leaves a factor
  2.5. Each step starts both methods from the oracle's positions, so one
  flipped decision does not carry over into later steps.
"""
import numpy as np
import pytest
import torch

from oracle import qmc_oracle as orc
from tests.golden_cases import load

pytestmark = pytest.mark.gpu

NW, NSTEP, STEP = 4096, 50, 0.2
TAU_MIXED = 1e-3


@pytest.fixture(scope="module")
def chain():
    mol, d = load("h2o_sd")
    ow = orc.OracleSlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"],
                                 fc_weight=d["fc_weight"].reshape(-1))
    rng = np.random.default_rng(4096)
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)
    pos0 = (centers[None] + rng.normal(size=(NW, mol.nelec, 3))).reshape(NW, -1)
    props = rng.normal(size=(NSTEP, NW, 3 * mol.nelec)) * orc.metropolis_sigma(STEP)
    unif = rng.uniform(size=(NSTEP, NW))
    trace = []
    samples, nacc, acc = orc.metropolis_replay(ow.pdf, pos0, props, unif, ntherm=0, ndecor=1,
                                               trace=trace)
    return dict(mol=mol, d=d, pos0=pos0, props=props, unif=unif,
                samples=samples.reshape(NSTEP, NW, -1), acc=np.asarray(acc), trace=trace,
                nacc=nacc)


def _wf(mol, d, precision):
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"], cuda=True,
                       precision=precision)
    wf.fc.weight.data = torch.as_tensor(d["fc_weight"], device="cuda").reshape(1, -1)
    return wf


def _sampler(mol, nstep):
    from qmctorch_gb300.sampler import Metropolis
    return Metropolis(nwalkers=NW, nstep=nstep, step_size=STEP, ntherm=0, ndecor=1,
                      nelec=mol.nelec, init=mol.domain("atomic"), cuda=True)


def test_fp64_chain_takes_every_decision_of_the_oracle(chain):
    mol, d = chain["mol"], chain["d"]
    wf = _wf(mol, d, "fp64")
    s = _sampler(mol, NSTEP)
    out = s(wf.pdf, pos=torch.as_tensor(chain["pos0"], device="cuda"), with_tqdm=False,
            replay={"proposals": chain["props"], "uniforms": chain["unif"]})
    snaps = out.detach().cpu().numpy().reshape(NSTEP, NW, -1)
    prev = np.concatenate([chain["pos0"][None], snaps[:-1]])
    gpu_acc = np.any(snaps != prev, axis=2)
    np.testing.assert_array_equal(gpu_acc, chain["acc"])
    np.testing.assert_allclose(snaps, chain["samples"], rtol=0, atol=1e-12)
    assert 0.1 < chain["acc"].mean() < 0.95  # a chain that moves and rejects


def test_mixed_decisions_differ_only_within_tolerance(chain):
    mol, d = chain["mol"], chain["d"]
    wf = _wf(mol, d, "mixed")
    flips, near, agree_pos_err = 0, 0, 0.0
    for k in range(NSTEP):
        x, ratio = chain["trace"][k]
        u = chain["unif"][k]
        s = _sampler(mol, 1)
        out = s(wf.pdf, pos=torch.as_tensor(x, device="cuda"), with_tqdm=False,
                replay={"proposals": chain["props"][k:k + 1], "uniforms": chain["unif"][k:k + 1]})
        new = out.detach().cpu().numpy()
        # the mixed method keeps positions as FP32 pairs (x to ~1e-14): a rejected
        # walker returns x to that accuracy, an accepted one moved by ~0.1 bohr
        gpu_acc = np.max(np.abs(new - x), axis=1) > 1e-9
        ref_acc = chain["acc"][k]
        margin = np.abs(ratio - u)
        flipped = gpu_acc != ref_acc
        near += int((margin < TAU_MIXED).sum())
        flips += int(flipped.sum())
        assert np.all(margin[flipped] < TAU_MIXED), (k, margin[flipped])
        same = ~flipped
        ref_new = chain["samples"][k]
        agree_pos_err = max(agree_pos_err, float(np.abs(new[same] - ref_new[same]).max()))
    assert agree_pos_err < 1e-12
    print("mixed replay: %d decisions, %d within tau=%g, %d flipped"
          % (NSTEP * NW, near, TAU_MIXED, flips))
