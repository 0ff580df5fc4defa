"""GPU tests of the hand-written adjoints of psi (qmc_wf_psi_adjoint behind
SlaterJastrow.forward's autograd function) and of the local energy
(qmc_wf_local_energy_adjoint behind SlaterJastrow.local_energy).

* Solver.evaluate_grad_manual reproduces the parameter gradients the
  reference computed with autograd (psi.backward(weight), solver.py:372-431)
  on the golden positions: 1e-8 relative (FP64; the adjoint sums walkers with
  atomic adds in no fixed order).
* Central finite differences (h = 1e-5) of sum_w g_w psi_w agree with the
  adjoint to 1e-6 relative.
* grad="auto" reproduces the reference's autograd gradient of mean(E_L)
  (solver.py:352-370) to 1e-8 relative; central differences of
  sum_w g_w E_L,w agree with the local-energy adjoint to 1e-5 relative.
"""
import numpy as np
import pytest
import torch

from tests.golden_cases import load

pytestmark = pytest.mark.gpu

PARAMS = ["ao.bas_exp", "mo.mo_modifier", "jastrow.jastrow_kernel.weight", "fc.weight"]


def make_wf(mol, d):
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"], cuda=True)
    wf.fc.weight.data = torch.as_tensor(d["fc_weight"], device="cuda").reshape(1, -1)
    return wf


@pytest.mark.parametrize("name", ["h2", "lih_cas", "lih_sd", "h2o_sd"])
def test_manual_gradient_matches_reference_autograd(name):
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.solver import Solver
    mol, d = load(name)
    wf = make_wf(mol, d)
    sampler = Metropolis(nwalkers=len(d["pos"]), nstep=2, step_size=0.2, nelec=mol.nelec,
                         init=mol.domain("atomic"), cuda=True)
    opt = torch.optim.Adam(wf.parameters(), lr=1e-3)
    solver = Solver(wf=wf, sampler=sampler, optimizer=opt)
    solver.configure(grad="manual", loss="energy", track=["local_energy"])
    solver.loss.use_weight = False
    opt.zero_grad()
    pos = torch.as_tensor(d["pos"], device="cuda")
    loss, eloc = solver.evaluate_gradient(pos)
    assert abs(float(loss) - float(d["grad_manual_loss"])) < 1e-9 * abs(float(d["grad_manual_loss"]))
    params = dict(wf.named_parameters())
    # gradients that vanish analytically (e.g. the single CI weight of a
    # ground-state wave function) are rounding noise on both sides: the
    # absolute floor is relative to the largest gradient of the case
    scale = max(np.abs(d["grad_manual_" + n]).max() for n in PARAMS)
    for n in PARAMS:
        ref = d["grad_manual_" + n]
        got = params[n].grad.detach().cpu().numpy().reshape(ref.shape)
        np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-12 * scale, err_msg=n)


@pytest.mark.parametrize("name", ["lih_cas", "h2o_sd"])
def test_adjoint_against_finite_differences(name):
    mol, d = load(name)
    wf = make_wf(mol, d)
    pos = torch.as_tensor(d["pos"], device="cuda")
    g = torch.as_tensor(np.random.default_rng(3).normal(size=len(d["pos"])), device="cuda")
    params = dict(wf.named_parameters())
    for p in params.values():
        p.grad = None
    (wf(pos).reshape(-1) * g).sum().backward()
    rng = np.random.default_rng(4)
    h = 1e-5
    with torch.no_grad():
        for n in PARAMS:
            p = params[n]
            flat = p.data.view(-1)
            picks = rng.choice(flat.numel(), size=min(4, flat.numel()), replace=False)
            for i in picks:
                i = int(i)
                old = float(flat[i])
                flat[i] = old + h
                fp = float((wf(pos).reshape(-1) * g).sum())
                flat[i] = old - h
                fm = float((wf(pos).reshape(-1) * g).sum())
                flat[i] = old
                fd = (fp - fm) / (2 * h)
                ad = float(p.grad.view(-1)[i])
                assert abs(fd - ad) <= 1e-6 * max(1.0, abs(fd)), (n, i, fd, ad)


def test_run_optimises_lih():
    """Solver.run (manual gradient, Adam) on LiH cas(2,2) lowers the energy."""
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.solver import Solver
    mol, d = load("lih_cas")
    wf = make_wf(mol, d)
    sampler = Metropolis(nwalkers=2048, nstep=200, step_size=0.2, nelec=mol.nelec,
                         init=mol.domain("atomic"), cuda=True, seed=5)
    opt = torch.optim.Adam(wf.parameters(), lr=1e-2)
    solver = Solver(wf=wf, sampler=sampler, optimizer=opt)
    obs = solver.run(15)
    e = np.asarray(obs.energy)
    assert np.all(np.isfinite(e)) and e[-3:].mean() < e[:3].mean()


@pytest.mark.parametrize("name", ["h2", "lih_cas", "lih_sd", "h2o_sd"])
def test_auto_gradient_matches_reference_autograd(name):
    """grad="auto": d mean(E_L) / d theta through the hand-written local-energy
    adjoint against the reference's autograd (solver.py:352-370), 1e-8 relative."""
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.solver import Solver
    mol, d = load(name)
    wf = make_wf(mol, d)
    sampler = Metropolis(nwalkers=len(d["pos"]), nstep=2, step_size=0.2, nelec=mol.nelec,
                         init=mol.domain("atomic"), cuda=True)
    opt = torch.optim.Adam(wf.parameters(), lr=1e-3)
    solver = Solver(wf=wf, sampler=sampler, optimizer=opt)
    solver.configure(grad="auto", loss="energy", track=["local_energy"])
    solver.loss.use_weight = False
    opt.zero_grad()
    pos = torch.as_tensor(d["pos"], device="cuda")
    loss, eloc = solver.evaluate_gradient(pos)
    assert abs(float(loss.detach()) - float(d["grad_auto_loss"])) < 1e-9 * abs(
        float(d["grad_auto_loss"]))
    params = dict(wf.named_parameters())
    scale = max(np.abs(d["grad_auto_" + n]).max() for n in PARAMS)
    for n in PARAMS:
        ref = d["grad_auto_" + n]
        got = params[n].grad.detach().cpu().numpy().reshape(ref.shape)
        np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-11 * scale, err_msg=n)


@pytest.mark.parametrize("name", ["lih_cas", "h2o_sd"])
def test_local_energy_adjoint_against_finite_differences(name):
    mol, d = load(name)
    wf = make_wf(mol, d)
    pos = torch.as_tensor(d["pos"], device="cuda")
    g = torch.as_tensor(np.random.default_rng(5).normal(size=len(d["pos"])), device="cuda")
    params = dict(wf.named_parameters())
    for p in params.values():
        p.grad = None
    (wf.local_energy(pos).reshape(-1) * g).sum().backward()
    rng = np.random.default_rng(6)
    h = 1e-5
    with torch.no_grad():
        for n in PARAMS:
            p = params[n]
            flat = p.data.view(-1)
            picks = rng.choice(flat.numel(), size=min(4, flat.numel()), replace=False)
            for i in picks:
                i = int(i)
                old = float(flat[i])
                flat[i] = old + h
                fp = float((wf.local_energy(pos).reshape(-1) * g).sum())
                flat[i] = old - h
                fm = float((wf.local_energy(pos).reshape(-1) * g).sum())
                flat[i] = old
                fd = (fp - fm) / (2 * h)
                ad = float(p.grad.view(-1)[i])
                assert abs(fd - ad) <= 1e-5 * max(1.0, abs(fd)), (n, i, fd, ad)


def test_gradients_are_bitwise_reproducible():
    """The adjoints sum walker contributions in a fixed order (no atomics):
    repeated backward passes give identical bits, for psi and for E_L."""
    mol, d = load("h2o_sd")
    wf = make_wf(mol, d)
    rng = np.random.default_rng(8)
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)
    pos = torch.as_tensor((centers[None] + rng.normal(size=(3000, 10, 3))).reshape(3000, -1),
                          device="cuda")
    g = torch.as_tensor(rng.normal(size=3000), device="cuda")
    params = dict(wf.named_parameters())
    for f in (lambda: wf(pos), lambda: wf.local_energy(pos)):
        grads = []
        for _ in range(2):
            for p in params.values():
                p.grad = None
            (f().reshape(-1) * g).sum().backward()
            grads.append([params[n].grad.detach().clone() for n in PARAMS])
        for a, b in zip(*grads):
            assert torch.equal(a, b)


@pytest.mark.parametrize("mode", ["manual", "auto"])
def test_single_precision_arm_matches_reference_fp32_autograd(mode):
    """The LiH cas(2,2) configuration in single precision: the reference run
    with torch's default dtype float32 (set_torch_single_precision,
    utils/torch_utils.py:16-21) against this package's mixed method on the
    same FP32 positions and CI weights. The reference's FP32 autograd itself
    differs from its FP64 run by ~1e-6 of the largest gradient; the bar is
    1e-4 of the largest gradient, and 1e-5 relative on the loss (the mixed
    local energies are within 5e-3 Ha per walker, their mean far closer)."""
    import os

    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.solver import Solver
    from tests.golden_cases import GOLDEN
    with np.load(os.path.join(GOLDEN, "lih_cas_fp32.npz")) as f:
        g32 = {k: f[k] for k in f.files}
    mol, d = load("lih_cas")
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"], cuda=True,
                       precision="mixed")
    wf.fc.weight.data = torch.as_tensor(g32["fc_weight32"].astype(np.float64),
                                        device="cuda").reshape(1, -1)
    pos = torch.as_tensor(g32["pos32"].astype(np.float64), device="cuda")
    sampler = Metropolis(nwalkers=len(pos), nstep=2, step_size=0.2, nelec=mol.nelec,
                         init=mol.domain("atomic"), cuda=True)
    opt = torch.optim.Adam(wf.parameters(), lr=1e-3)
    solver = Solver(wf=wf, sampler=sampler, optimizer=opt)
    solver.configure(grad=mode, loss="energy", track=["local_energy"])
    solver.loss.use_weight = False
    opt.zero_grad()
    loss, _ = solver.evaluate_gradient(pos)
    ref_loss = float(g32["grad32_%s_loss" % mode])
    assert abs(float(loss.detach()) - ref_loss) < 1e-5 * abs(ref_loss)
    params = dict(wf.named_parameters())
    scale = max(np.abs(g32["grad32_%s_%s" % (mode, n)]).max() for n in PARAMS)
    for n in PARAMS:
        ref = g32["grad32_%s_%s" % (mode, n)]
        got = params[n].grad.detach().cpu().numpy().reshape(ref.shape)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-4 * scale, err_msg=n)
