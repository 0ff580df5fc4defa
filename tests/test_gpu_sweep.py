"""GPU tests of the single-electron sampler with Sherman-Morrison updates
(qmc_sweep.cu), used by qmc_metropolis_run for one-elec and all-elec-iter
moves of a single ground-state determinant.

* With the reference's proposals, uniforms and electron indices replayed, the
  positions match the reference's own run (golden fixtures of h4 and c6h6):
  1e-12 relative in FP64, 1e-9 in the mixed method (positions are FP32 pairs).
* With generated random numbers the sweep kernel and the generic kernel (full
  re-evaluation per move, forced through the C ABI by requesting psi_out) take
  the same decisions: identical chains in FP64; in the mixed method at least
  95 % of the walkers end identical (a decision flips only where the FP32
  ratio and the uniform agree to ~1e-5).
"""
import ctypes

import numpy as np
import pytest
import torch

from tests.golden_cases import load

pytestmark = pytest.mark.gpu


def make_wf(mol, d, precision):
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"], cuda=True,
                       precision=precision)
    wf.fc.weight.data = torch.as_tensor(d["fc_weight"], device="cuda").reshape(1, -1)
    return wf


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("mixed", 1e-9)])
@pytest.mark.parametrize("name", ["h4", "c6h6"])
def test_iter_replay_matches_reference(name, precision, rtol):
    from qmctorch_gb300.sampler import Metropolis
    mol, d = load(name)
    wf = make_wf(mol, d, precision)
    props, unif = d["iter_props"], d["iter_unif"]
    nstep, nw = unif.shape[0], unif.shape[2]
    s = Metropolis(nwalkers=nw, nstep=nstep, step_size=0.3, ntherm=-1, ndecor=1, nelec=mol.nelec,
                   init=mol.domain("atomic"), move={"type": "all-elec-iter", "proba": "normal"},
                   cuda=True)
    out = s(wf.pdf, pos=torch.as_tensor(d["iter_pos0"], device="cuda"), with_tqdm=False,
            replay={"proposals": props, "uniforms": unif})
    np.testing.assert_allclose(out.detach().cpu().numpy(), d["iter_out"], rtol=rtol, atol=1e-12)


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("mixed", 1e-9)])
@pytest.mark.parametrize("name", ["h4", "c6h6"])
def test_one_elec_replay_matches_reference(name, precision, rtol):
    from qmctorch_gb300.sampler import Metropolis
    mol, d = load(name)
    wf = make_wf(mol, d, precision)
    nstep, nw = d["one_unif"].shape
    s = Metropolis(nwalkers=nw, nstep=nstep, step_size=float(d["one_step"]),
                   ntherm=int(d["one_ntherm"]), ndecor=int(d["one_ndecor"]), nelec=mol.nelec,
                   init=mol.domain("atomic"), move={"type": "one-elec", "proba": "normal"},
                   cuda=True)
    out = s(wf.pdf, pos=torch.as_tensor(d["one_pos0"], device="cuda"), with_tqdm=False,
            replay={"proposals": d["one_props"], "uniforms": d["one_unif"],
                    "electron_index": d["one_index"]})
    np.testing.assert_allclose(out.detach().cpu().numpy(), d["one_out"], rtol=rtol, atol=1e-12)


def _run_capi(wf, x, nstep, move_type, seed, generic):
    """qmc_metropolis_run on x (advanced in place); generic=True requests
    psi_out, which routes the call to the full re-evaluation kernel."""
    from qmctorch_gb300 import _lib
    from qmctorch_gb300.wavefunction import runtime as rt
    lib = _lib.lib()
    nw = x.shape[0]
    call = wf._desc(x.device)
    need = lib.qmc_metropolis_scratch_bytes(call.ref, nw)
    scr = torch.empty(max(need, 1), dtype=torch.uint8, device=x.device)
    psi = torch.empty(nw, dtype=torch.float64, device=x.device)
    acc = torch.zeros(nw, dtype=torch.int32, device=x.device)
    a = _lib.MetropolisArgs()
    a.pos = rt.ptr(x)
    a.nwalkers = nw
    a.nstep = nstep
    a.ntherm = nstep
    a.ndecor = 1
    a.move_type = move_type
    a.proba = 0
    a.step_size = 0.2
    a.seed = seed
    a.step_offset = 0
    a.samples = None
    a.nsnap = 0
    a.accepted = rt.ptr(acc)
    a.psi_out = rt.ptr(psi) if generic else None
    st = lib.qmc_metropolis_run(call.ref, a, rt.ptr(scr), scr.numel(), rt.stream_handle())
    assert st == 0, lib.qmc_status_string(st)
    torch.cuda.synchronize()
    return acc.cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("move_type", [1, 2])  # QMC_MOVE_ONE_ELEC, QMC_MOVE_ALL_ELEC_ITER
def test_sweep_kernel_matches_generic_kernel(precision, move_type):
    mol, d = load("c6h6")
    wf = make_wf(mol, d, precision)
    rng = np.random.default_rng(5)
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)
    nw = 256
    x0 = torch.as_tensor((centers[None] + 0.7 * rng.normal(size=(nw, mol.nelec, 3)))
                         .reshape(nw, -1), device="cuda")
    nstep = 3 if move_type == 2 else 60
    xs, xg = x0.clone(), x0.clone()
    acc_s = _run_capi(wf, xs, nstep, move_type, 77, generic=False)
    acc_g = _run_capi(wf, xg, nstep, move_type, 77, generic=True)
    assert acc_s.sum() > 0
    same = (xs == xg).all(dim=1).cpu().numpy()
    if precision == "fp64":
        assert same.all()
        np.testing.assert_array_equal(acc_s, acc_g)
    else:
        assert same.mean() >= 0.95, same.mean()
