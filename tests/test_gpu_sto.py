"""GPU parity of Slater-type orbitals (ADF layout: radial_type "sto",
cartesian harmonics, r^kr exp(-a r); radial_functions.py:6-123,
atomic_orbitals.py:15-423, norm_orbital.py:106-161) against outputs of the
reference itself (golden fixtures lih_sto, h2o_sto in the "slater-sz" basis).

Tolerances are those of the Gaussian cases: FP64 1e-10 relative on the AO
values and derivatives, psi, E_L and gradients (absolute floor 1e-12 of the
largest magnitude); Metropolis replays 1e-12; parameter gradients (including
d/d exponent of the Slater primitives) 1e-8 relative to the reference's
autograd; the mixed method 1e-4 relative on psi and 5e-3 Ha on E_L.
"""
import numpy as np
import pytest
import torch

from tests.golden_cases import STO_CASES, load, make_wf

pytestmark = pytest.mark.gpu

RTOL = 1e-10
PARAMS = ["ao.bas_exp", "mo.mo_modifier", "jastrow.jastrow_kernel.weight", "fc.weight"]


def close(a, b, rtol=RTOL, floor=1e-12):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    atol = floor * max(1.0, float(np.abs(b).max()))
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


@pytest.mark.parametrize("name", STO_CASES)
def test_atomic_orbitals(name):
    mol, d = load(name)
    wf = make_wf(mol, d)
    pos = torch.as_tensor(d["pos"]).cuda()
    ao, dao, d2ao = wf.ao(pos, derivative=[0, 1, 2])
    close(ao, d["ao"])
    close(dao, d["dao"])
    close(d2ao, d["d2ao"])
    close(wf.ao(pos, derivative=1), d["ao_sumgrad"])
    close(wf.mo(ao), d["mo"])


@pytest.mark.parametrize("name", STO_CASES)
def test_psi_local_energy_and_gradients(name):
    mol, d = load(name)
    wf = make_wf(mol, d)
    pos = torch.as_tensor(d["pos"]).cuda()
    close(wf(pos), d["psi"])
    close(wf.pdf(pos), d["pdf"])
    close(wf.kinetic_energy(pos), d["kinetic"])
    close(wf.local_energy(pos), d["eloc"])
    close(wf.gradients_jacobi(pos), d["grad_psi"])


@pytest.mark.parametrize("name", STO_CASES)
def test_mixed_method(name):
    mol, d = load(name)
    wf = make_wf(mol, d, precision="mixed")
    pos = torch.as_tensor(d["pos"]).cuda()
    psi = wf(pos).detach().cpu().numpy().ravel()
    assert np.max(np.abs(psi - d["psi"].ravel()) / np.abs(d["psi"].ravel())) <= 1e-4
    el = wf.local_energy(pos).detach().cpu().numpy().ravel()
    assert np.max(np.abs(el - d["eloc"].ravel())) <= 5e-3


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("mixed", 1e-9)])
@pytest.mark.parametrize("name", STO_CASES)
def test_metropolis_replay(name, precision, rtol):
    from qmctorch_gb300.sampler import Metropolis
    mol, d = load(name)
    wf = make_wf(mol, d, precision=precision)
    props, unif = d["met_props"], d["met_unif"]
    nstep, nw = unif.shape
    s = Metropolis(nwalkers=nw, nstep=nstep, step_size=float(d["met_step"]),
                   ntherm=int(d["met_ntherm"]), ndecor=int(d["met_ndecor"]), nelec=mol.nelec,
                   init=mol.domain("atomic"), cuda=True)
    out = s(wf.pdf, pos=torch.as_tensor(d["met_pos0"]).cuda(), with_tqdm=False,
            replay={"proposals": props, "uniforms": unif})
    close(out, d["met_out"], rtol=rtol)


@pytest.mark.parametrize("mode", ["manual", "auto"])
@pytest.mark.parametrize("name", STO_CASES)
def test_parameter_gradients_match_reference_autograd(name, mode):
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.solver import Solver
    mol, d = load(name)
    wf = make_wf(mol, d)
    sampler = Metropolis(nwalkers=len(d["pos"]), nstep=2, step_size=0.2, nelec=mol.nelec,
                         init=mol.domain("atomic"), cuda=True)
    opt = torch.optim.Adam(wf.parameters(), lr=1e-3)
    solver = Solver(wf=wf, sampler=sampler, optimizer=opt)
    solver.configure(grad=mode, loss="energy", track=["local_energy"])
    solver.loss.use_weight = False
    opt.zero_grad()
    loss, _ = solver.evaluate_gradient(torch.as_tensor(d["pos"], device="cuda"))
    ref_loss = float(d["grad_%s_loss" % mode])
    assert abs(float(loss.detach()) - ref_loss) < 1e-9 * abs(ref_loss)
    params = dict(wf.named_parameters())
    scale = max(np.abs(d["grad_%s_%s" % (mode, n)]).max() for n in PARAMS)
    for n in PARAMS:
        ref = d["grad_%s_%s" % (mode, n)]
        got = params[n].grad.detach().cpu().numpy().reshape(ref.shape)
        np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-11 * scale, err_msg=n)
