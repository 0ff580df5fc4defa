"""GPU tests of the mixed-precision method (FP32 AO / AO->MO / Jastrow / LU
with FP64 determinant products, sums and refinement) against the FP64
reference values.

Stated tolerances (per walker, on the golden positions of every case):
psi relative error <= 1e-4, kinetic energy relative error <= 2e-4,
local-energy absolute error <= 5e-3 Ha. On 1e5 fixed H2O positions the mean
local energy must agree with the FP64 method within 1e-5 Ha.
"""
import numpy as np
import pytest
import torch

from tests.golden_cases import CASES, load

pytestmark = pytest.mark.gpu


def make_wf(mol, d, precision):
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"], cuda=True,
                       precision=precision)
    wf.fc.weight.data = torch.as_tensor(d["fc_weight"], device="cuda").reshape(1, -1)
    return wf


@pytest.mark.parametrize("name", CASES)
def test_mixed_against_reference_values(name):
    mol, d = load(name)
    wf = make_wf(mol, d, "mixed")
    x = torch.as_tensor(d["pos"], device="cuda")
    psi = wf(x).detach().cpu().numpy().ravel()
    ref = d["psi"].ravel()
    assert np.max(np.abs(psi - ref) / np.abs(ref)) <= 1e-4
    kin = wf.kinetic_energy(x).cpu().numpy().ravel()
    assert np.max(np.abs(kin - d["kinetic"].ravel()) / np.abs(d["kinetic"].ravel())) <= 2e-4
    el = wf.local_energy(x).detach().cpu().numpy().ravel()
    assert np.max(np.abs(el - d["eloc"].ravel())) <= 5e-3
    pdf = wf.pdf(x).cpu().numpy()
    assert np.max(np.abs(pdf - d["pdf"]) / np.abs(d["pdf"])) <= 2e-4


def test_mixed_mean_local_energy_on_fixed_positions():
    """H2O cc-pVDZ single_double(4,4): mean E_L of the mixed method on 1e5
    equilibrated positions within 1e-5 Ha of the FP64 method (which matches
    the reference to 1e-10 relative)."""
    from qmctorch_gb300.sampler import Metropolis
    mol, d = load("h2o_sd")
    wf64 = make_wf(mol, d, "fp64")
    wfm = make_wf(mol, d, "mixed")
    rng = np.random.default_rng(1234)
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)
    x = torch.as_tensor((centers[None] + rng.normal(size=(16384, 10, 3))).reshape(16384, -1),
                        device="cuda")
    s = Metropolis(nwalkers=16384, nstep=10, step_size=0.2, nelec=10, init=mol.domain("atomic"),
                   cuda=True, seed=1234)
    s.advance(wf64.pdf, x, nstep=600)
    snaps = []
    for _ in range(7):
        s.advance(wf64.pdf, x, nstep=10)
        snaps.append(x.clone())
    X = torch.cat(snaps)[:100000]
    with torch.no_grad():
        e64 = wf64.local_energy(X).double()
        em = wfm.local_energy(X).double()
    assert abs(float(em.mean() - e64.mean())) < 1e-5
    with torch.no_grad():
        psi_err = ((wfm(X) - wf64(X)) / wf64(X)).abs()
    assert float(psi_err.median()) < 1e-5


@pytest.mark.parametrize("name", ["h2", "h2o_sd"])
def test_mixed_metropolis_replay_decisions(name):
    """With the reference's proposals and uniforms, the mixed sampler takes
    the same accept/reject decisions (no |ratio - u| near-tie occurs in these
    fixtures) and so keeps the same positions."""
    from qmctorch_gb300.sampler import Metropolis
    mol, d = load(name)
    wf = make_wf(mol, d, "mixed")
    props, unif = d["met_props"], d["met_unif"]
    nstep, nw = unif.shape
    sampler = Metropolis(nwalkers=nw, nstep=nstep, step_size=float(d["met_step"]),
                         ntherm=int(d["met_ntherm"]), ndecor=int(d["met_ndecor"]), nelec=mol.nelec,
                         init=mol.domain("atomic"), cuda=True)
    out = sampler(wf.pdf, pos=torch.as_tensor(d["met_pos0"], device="cuda"), with_tqdm=False,
                  replay={"proposals": props, "uniforms": unif})
    np.testing.assert_allclose(out.detach().cpu().numpy(), d["met_out"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_size_does_not_change_results(precision):
    """The launch plan (walkers per block, threads per walker) depends on the
    batch size; each walker's arithmetic does not. psi, E_L and a Metropolis
    chain of the first 64 walkers are bitwise the same alone and inside a
    batch of 16384."""
    from qmctorch_gb300.sampler import Metropolis
    mol, d = load("h2o_sd")
    wf = make_wf(mol, d, precision)
    rng = np.random.default_rng(77)
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)
    big = torch.as_tensor((centers[None] + rng.normal(size=(16384, 10, 3))).reshape(16384, -1),
                          device="cuda")
    small = big[:64].clone()
    with torch.no_grad():
        np.testing.assert_array_equal(wf(small).cpu().numpy(), wf(big)[:64].cpu().numpy())
    with torch.no_grad():
        np.testing.assert_array_equal(wf.local_energy(small).cpu().numpy(),
                                      wf.local_energy(big)[:64].cpu().numpy())
    outs = []
    for x in (small, big):
        s = Metropolis(nwalkers=len(x), nstep=30, step_size=0.2, nelec=10,
                       init=mol.domain("atomic"), cuda=True, seed=9)
        outs.append(s(wf.pdf, pos=x.clone(), with_tqdm=False)[:64].detach().cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_large_chain_plan_does_not_change_results(precision):
    """H20 sto-3g at 16384 walkers has no one-wave launch plan with the
    current positions in shared memory; the mixed method's plan keeps them in
    the scratch instead (one wave). A chain of the first 64 walkers (whose plan keeps them in shared
    memory) is bitwise the same as inside the 16384-walker batch."""
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.scf import Molecule
    from qmctorch_gb300.serving import hydrogen_chain, seeded_positions
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    mol = Molecule(hydrogen_chain(20, 0.95), unit="angs", basis="sto-3g", calculator="huckel")
    wf = SlaterJastrow(mol, cuda=True, precision=precision)
    big = torch.as_tensor(seeded_positions(mol, 16384, seed=20), device="cuda")
    small = big[:64].clone()
    import ctypes

    from qmctorch_gb300 import _lib
    call = wf._desc(torch.device("cuda"))
    plans = {}
    for nw in (64, 16384):
        plan = (ctypes.c_int32 * 5)()
        assert _lib.lib().qmc_metropolis_plan(call.ref, nw, plan) == 0
        plans[nw] = list(plan)
    assert plans[64][3] == 0, plans
    if precision == "mixed":  # one wave: 4 blocks of 32 walkers per SM
        assert plans[16384][3] == 1 and 152 * 4 * plans[16384][0] >= 16384, plans
    print("H20 %s plans (nwb, nslot, threads, pos in scratch, smem):" % precision, plans)
    outs = []
    for x in (small, big):
        s = Metropolis(nwalkers=len(x), nstep=12, step_size=0.2, nelec=mol.nelec,
                       init=mol.domain("atomic"), cuda=True, seed=21)
        outs.append(s(wf.pdf, pos=x.clone(), with_tqdm=False)[:64].detach().cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
    assert np.isfinite(outs[1]).all()
