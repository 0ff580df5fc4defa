"""GPU parity of the electron-nucleus Pade Jastrow factor, alone ("en") and
combined with the e-e factor ("ee+en", CombineJastrow), against outputs of the
reference itself (golden fixtures h2_en, lih_en, h2o_en, c6h6_en;
jastrow_factor_electron_nuclei.py:9-161, elec_nuclei/kernels/
pade_jastrow_kernel.py:8-116, combine_jastrow.py:7-195).

Tolerances are those of the e-e cases: FP64 1e-10 relative on psi, E_L,
gradients and the module outputs (absolute floor 1e-12 of the largest
magnitude); Metropolis replays 1e-12; parameter gradients 1e-8 relative to the
reference's autograd; the mixed method 1e-4 relative on psi and 5e-3 Ha on E_L.
"""
import numpy as np
import pytest
import torch

from oracle import qmc_oracle as orc
from tests.golden_cases import EN_CASES, jastrow_weights, load, make_wf, param_names

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def close(a, b, rtol=RTOL, floor=1e-12):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    atol = floor * max(1.0, float(np.abs(b).max()))
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


@pytest.mark.parametrize("name", EN_CASES)
def test_psi_local_energy_and_gradients(name):
    mol, d = load(name)
    wf = make_wf(mol, d)
    pos = torch.as_tensor(d["pos"]).cuda()
    close(wf(pos), d["psi"])
    close(wf.pdf(pos), d["pdf"])
    close(wf.kinetic_energy(pos), d["kinetic"])
    close(wf.local_energy(pos), d["eloc"])
    close(wf.gradients_jacobi(pos), d["grad_psi"])
    close(wf.pdf(pos, return_grad=True), d["grad_pdf"])


@pytest.mark.parametrize("name", [c for c in EN_CASES if not c.startswith("c6h6")])
def test_jastrow_modules(name):
    """The standalone Jastrow module call (e-n factor, or CombineJastrow of
    the e-e and e-n factors) against the reference's J, grad J, lap J."""
    mol, d = load(name)
    wf = make_wf(mol, d)
    pos = torch.as_tensor(d["pos"]).cuda()
    j, dj, d2j = wf.jastrow(pos, derivative=[0, 1, 2], sum_grad=False)
    close(j, d["jast"])
    close(dj, d["djast"])
    close(d2j, d["d2jast"])
    close(wf.jastrow(pos), d["jast"])
    close(wf.jastrow(pos, derivative=1), d["djast_sum"])
    close(wf.jastrow(pos, derivative=1, sum_grad=False), d["djast"])
    close(wf.jastrow(pos, derivative=2), d["d2jast"])


@pytest.mark.parametrize("name", EN_CASES)
def test_matches_oracle_on_fresh_positions(name):
    mol, d = load(name)
    wf = make_wf(mol, d)
    ow = orc.OracleSlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"],
                                 jastrow_terms=jastrow_weights(d), fc_weight=d["fc_weight"])
    rng = np.random.default_rng(98)
    nw = 4 if name.startswith("c6h6") else 37
    pos = d["pos"][rng.integers(0, len(d["pos"]), nw)] + 0.3 * rng.normal(
        size=(nw, d["pos"].shape[1]))
    x = torch.as_tensor(pos).cuda()
    close(wf(x), ow.forward(pos), rtol=1e-9)
    close(wf.local_energy(x), ow.local_energy(pos), rtol=1e-9)


@pytest.mark.parametrize("name", EN_CASES)
def test_mixed_method(name):
    mol, d = load(name)
    wf = make_wf(mol, d, precision="mixed")
    pos = torch.as_tensor(d["pos"]).cuda()
    psi = wf(pos).detach().cpu().numpy().ravel()
    assert np.max(np.abs(psi - d["psi"].ravel()) / np.abs(d["psi"].ravel())) <= 1e-4
    el = wf.local_energy(pos).detach().cpu().numpy().ravel()
    assert np.max(np.abs(el - d["eloc"].ravel())) <= 5e-3


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("mixed", 1e-9)])
@pytest.mark.parametrize("name", [c for c in EN_CASES if "met_out" in load(c)[1]])
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


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("mixed", 1e-9)])
@pytest.mark.parametrize("name", [c for c in EN_CASES if "iter_out" in load(c)[1]])
def test_iter_replay(name, precision, rtol):
    """all-elec-iter moves: c6h6_en (one determinant) runs the
    Sherman-Morrison sweep kernel, h2o_en the re-evaluating kernel."""
    from qmctorch_gb300.sampler import Metropolis
    mol, d = load(name)
    wf = make_wf(mol, d, precision=precision)
    props, unif = d["iter_props"], d["iter_unif"]
    nstep, nw = unif.shape[0], unif.shape[2]
    s = Metropolis(nwalkers=nw, nstep=nstep, step_size=0.3, ntherm=-1, ndecor=1, nelec=mol.nelec,
                   init=mol.domain("atomic"), move={"type": "all-elec-iter", "proba": "normal"},
                   cuda=True)
    out = s(wf.pdf, pos=torch.as_tensor(d["iter_pos0"], device="cuda"), with_tqdm=False,
            replay={"proposals": props, "uniforms": unif})
    np.testing.assert_allclose(out.detach().cpu().numpy(), d["iter_out"], rtol=rtol, atol=1e-12)


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("mixed", 1e-9)])
def test_one_elec_replay_sweep_kernel(precision, rtol):
    from qmctorch_gb300.sampler import Metropolis
    mol, d = load("c6h6_en")
    wf = make_wf(mol, d, precision=precision)
    nstep, nw = d["one_unif"].shape
    s = Metropolis(nwalkers=nw, nstep=nstep, step_size=float(d["one_step"]),
                   ntherm=int(d["one_ntherm"]), ndecor=int(d["one_ndecor"]), nelec=mol.nelec,
                   init=mol.domain("atomic"), move={"type": "one-elec", "proba": "normal"},
                   cuda=True)
    out = s(wf.pdf, pos=torch.as_tensor(d["one_pos0"], device="cuda"), with_tqdm=False,
            replay={"proposals": d["one_props"], "uniforms": d["one_unif"],
                    "electron_index": d["one_index"]})
    np.testing.assert_allclose(out.detach().cpu().numpy(), d["one_out"], rtol=rtol, atol=1e-12)


@pytest.mark.parametrize("mode", ["manual", "auto"])
@pytest.mark.parametrize("name", [c for c in EN_CASES if "grad_manual_loss" in load(c)[1]])
def test_parameter_gradients_match_reference_autograd(name, mode):
    """Solver gradients through the hand-written adjoints (psi for "manual",
    E_L for "auto") against the reference's autograd on the golden positions,
    including d/dw of both Pade weights."""
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
    pos = torch.as_tensor(d["pos"], device="cuda")
    loss, _ = solver.evaluate_gradient(pos)
    ref_loss = float(d["grad_%s_loss" % mode])
    assert abs(float(loss.detach()) - ref_loss) < 1e-9 * abs(ref_loss)
    names = ["ao.bas_exp", "mo.mo_modifier", "fc.weight"] + param_names(d)
    params = dict(wf.named_parameters())
    scale = max(np.abs(d["grad_%s_%s" % (mode, n)]).max() for n in names)
    for n in names:
        ref = d["grad_%s_%s" % (mode, n)]
        got = params[n].grad.detach().cpu().numpy().reshape(ref.shape)
        np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-11 * scale, err_msg=n)


def test_en_weight_gradient_against_finite_differences():
    """d/dw_en of sum_w g_w psi_w and of sum_w g_w E_L,w by the adjoints
    against central differences (h = 1e-5), on H2O cc-pVDZ ee+en."""
    mol, d = load("h2o_en")
    wf = make_wf(mol, d)
    pos = torch.as_tensor(d["pos"], device="cuda")
    g = torch.as_tensor(np.random.default_rng(3).normal(size=len(d["pos"])), device="cuda")
    p = dict(wf.named_parameters())[param_names(d)[-1]]
    h = 1e-5
    for f, tol in ((lambda: wf(pos).reshape(-1), 1e-6), (lambda: wf.local_energy(pos).reshape(-1),
                                                         1e-5)):
        p.grad = None
        (f() * g).sum().backward()
        ad = float(p.grad[0])
        with torch.no_grad():
            old = float(p.data[0])
            p.data[0] = old + h
            fp = float((f() * g).sum())
            p.data[0] = old - h
            fm = float((f() * g).sum())
            p.data[0] = old
        fd = (fp - fm) / (2 * h)
        assert abs(fd - ad) <= tol * max(1.0, abs(fd)), (fd, ad)
