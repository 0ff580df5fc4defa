"""GPU tests of the serving path: the batched Metropolis launch, the
compensated statistics kernel and the continuous-batching server.

* qmc_metropolis_run_batch advances every job bitwise as qmc_metropolis_run
  does alone, with molecules of different sizes in one launch; jobs of
  different precisions are refused (QMC_ERR_SHAPE).
* qmc_reduce_stats: mean within 1e-15 and variance within 1e-13 relative of an
  exactly rounded reference (math.fsum), n = 1 gives a NaN variance as
  torch.var does.
* A request's result (energy, variance, error) is bitwise the same served
  alone and served in a mix of requests of other sizes that arrive while it
  runs, and equals sampling + local energy + statistics done by hand.
"""
import ctypes
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _mol(n, spacing):
    from qmctorch_gb300.scf import Molecule
    from qmctorch_gb300.serving import hydrogen_chain
    return Molecule(hydrogen_chain(n, spacing), unit="angs", basis="sto-3g", calculator="huckel")


def _wf(mol, precision="mixed"):
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    return SlaterJastrow(mol, configs="ground_state", cuda=True, precision=precision)


def _args(x, nstep, seed, offset=0):
    from qmctorch_gb300 import _lib
    a = _lib.MetropolisArgs()
    a.pos = ctypes.c_void_p(x.data_ptr())
    a.nwalkers, a.nstep, a.ntherm, a.ndecor = x.shape[0], nstep, nstep, 1
    a.move_type, a.proba, a.step_size, a.seed, a.step_offset = 0, 0, 0.2, seed, offset
    return a


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_launch_matches_single_launches(precision):
    from qmctorch_gb300 import _lib
    from qmctorch_gb300.serving import seeded_positions
    lib = _lib.lib()
    # molecules of different sizes share the launch (one MO column class)
    jobs = [(_mol(4, 0.74), 700, 11), (_mol(10, 0.95), 1500, 12), (_mol(6, 1.2), 33, 13),
            (_mol(16, 0.9), 257, 14)]
    wfs = [_wf(m, precision) for m, _, _ in jobs]
    x0 = [torch.as_tensor(seeded_positions(m, nw, s), device="cuda") for m, nw, s in jobs]
    # alone
    alone = []
    for wf, x, (m, nw, seed) in zip(wfs, x0, jobs):
        x = x.clone()
        call = wf._desc(x.device)
        scr = torch.empty(lib.qmc_metropolis_scratch_bytes(call.ref, nw), dtype=torch.uint8,
                          device="cuda")
        a = _args(x, 40, seed, offset=5)
        _lib.check(lib.qmc_metropolis_run(call.ref, a, ctypes.c_void_p(scr.data_ptr()),
                                          scr.numel(), None), "run")
        alone.append(x)
    # batched
    xs = [x.clone() for x in x0]
    calls = [wf._desc(x.device) for wf, x in zip(wfs, xs)]
    scrs = [torch.empty(lib.qmc_metropolis_scratch_bytes(c.ref, x.shape[0]), dtype=torch.uint8,
                        device="cuda") for c, x in zip(calls, xs)]
    n = len(jobs)
    descs = (_lib.WfDesc * n)(*[c.desc for c in calls])
    args = (_lib.MetropolisArgs * n)(*[_args(x, 40, s, offset=5) for x, (_, _, s) in zip(xs, jobs)])
    sp = (ctypes.c_void_p * n)(*[s.data_ptr() for s in scrs])
    nb = (ctypes.c_int64 * n)(*[s.numel() for s in scrs])
    _lib.check(lib.qmc_metropolis_run_batch(descs, args, sp, nb, n, None), "batch")
    torch.cuda.synchronize()
    for xa, xb in zip(alone, xs):
        assert torch.equal(xa, xb)
    # a job of another precision is refused
    other = _wf(_mol(6, 0.74), "fp64" if precision == "mixed" else "mixed")
    c6 = other._desc(torch.device("cuda"))
    x6 = torch.as_tensor(seeded_positions(other.mol, 64, 1), device="cuda")
    s6 = torch.empty(lib.qmc_metropolis_scratch_bytes(c6.ref, 64), dtype=torch.uint8, device="cuda")
    descs2 = (_lib.WfDesc * 2)(calls[0].desc, c6.desc)
    args2 = (_lib.MetropolisArgs * 2)(_args(xs[0], 1, 1), _args(x6, 1, 1))
    sp2 = (ctypes.c_void_p * 2)(scrs[0].data_ptr(), s6.data_ptr())
    nb2 = (ctypes.c_int64 * 2)(scrs[0].numel(), s6.numel())
    assert lib.qmc_metropolis_run_batch(descs2, args2, sp2, nb2, 2, None) == 2


def _stats(x):
    from qmctorch_gb300 import _lib
    lib = _lib.lib()
    n = x.numel()
    scr = torch.empty(lib.qmc_reduce_scratch_bytes(n), dtype=torch.uint8, device="cuda")
    out = torch.empty(3, dtype=torch.float64, device="cuda")
    _lib.check(lib.qmc_reduce_stats(ctypes.c_void_p(x.data_ptr()), n,
                                    ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(scr.data_ptr()), scr.numel(), None), "stats")
    return out.cpu().tolist()


@pytest.mark.parametrize("n", [1, 2, 777, 100003, 3000000])
def test_reduce_stats_against_exact_sums(n):
    rng = np.random.default_rng(n)
    v = -70.7 + 0.3 * rng.standard_normal(n)
    mean, var, err = _stats(torch.as_tensor(v, device="cuda"))
    m = math.fsum(v) / n
    assert abs(mean - m) <= 1e-15 * abs(m)
    if n == 1:
        assert math.isnan(var)
        return
    d = v - m
    ref = (math.fsum(d * d) - math.fsum(d) ** 2 / n) / (n - 1)
    assert abs(var - ref) <= 1e-13 * ref
    assert abs(err - math.sqrt(ref / n)) <= 1e-13 * math.sqrt(ref / n)


def _requests():
    from qmctorch_gb300.serving import Request, hydrogen_chain
    rng = np.random.default_rng(0)
    out = []
    for i in range(9):
        n = int(rng.choice([2, 4, 6, 8]))
        out.append(Request(atoms=hydrogen_chain(n, float(rng.uniform(0.7, 1.2))),
                           nwalkers=int(rng.integers(512, 3000)),
                           nstep=int(rng.integers(60, 240)), seed=100 + i))
    return out


def test_result_is_the_same_alone_and_in_the_mix():
    import copy

    from qmctorch_gb300.serving import VMCServer, single_point
    reqs = _requests()
    srv = VMCServer(hbm_budget=256 << 20, slice_steps=32)  # not every request fits at once
    for r in reqs[:4]:
        srv.submit(copy.copy(r))
    for _ in range(3):
        srv.poll()
    for r in reqs[4:]:  # arrive while the first ones run
        srv.submit(copy.copy(r))
    srv.run()
    assert srv.launched_jobs > srv.launches  # requests of different sizes shared launches
    for rid, r in enumerate(reqs):
        mixed = srv.results[rid]
        alone = single_point(copy.copy(r))
        assert (mixed.energy, mixed.variance, mixed.error) == (alone.energy, alone.variance,
                                                                alone.error)
        assert np.isfinite(mixed.energy) and mixed.variance > 0


def test_single_point_equals_sampling_by_hand():
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.serving import Request, hydrogen_chain, seeded_positions, single_point
    r = Request(atoms=hydrogen_chain(6, 0.9), nwalkers=2048, nstep=150, seed=7, precision="fp64")
    res = single_point(r)
    mol = _mol(6, 0.9)
    wf = _wf(mol, "fp64")
    x = torch.as_tensor(seeded_positions(mol, r.nwalkers, r.seed), device="cuda")
    s = Metropolis(nwalkers=r.nwalkers, nstep=r.nstep, step_size=r.step_size, nelec=mol.nelec,
                   init=mol.domain("atomic"), cuda=True, seed=r.seed)
    s.advance(wf.pdf, x, nstep=r.nstep)
    el = wf.local_energy(x).reshape(-1).detach().cpu().numpy()
    m = math.fsum(el) / len(el)
    var = float(np.var(el, ddof=1))
    assert abs(res.energy - m) <= 1e-14 * abs(m)
    assert abs(res.variance - var) <= 1e-10 * var
    assert abs(res.error - math.sqrt(var / len(el))) <= 1e-10 * math.sqrt(var / len(el))


def test_run_request_is_the_same_alone_and_in_the_mix():
    """VMC-run jobs (gradient through the psi adjoint with a fixed-order
    reduction, Adam, resampling) are bitwise reproducible: alone and among
    single points of other sizes give the same epoch energies and result."""
    import copy

    from qmctorch_gb300.serving import Request, VMCServer, hydrogen_chain, single_point
    run = Request(atoms=hydrogen_chain(4, 0.95), nwalkers=1536, nstep=80, seed=21, kind="run",
                  nepoch=6, lr=1e-2, nstep_update=20)
    others = [r for r in _requests()[:5]]
    srv = VMCServer(hbm_budget=1 << 30, slice_steps=32)
    srv.submit(copy.copy(others[0]))
    rid = srv.submit(copy.copy(run))
    srv.poll()
    for r in others[1:]:
        srv.submit(copy.copy(r))
    srv.run()
    mixed = srv.results[rid]
    alone = single_point(copy.copy(run))
    assert mixed.energies == alone.energies and len(mixed.energies) == 6
    assert (mixed.energy, mixed.variance, mixed.error) == (alone.energy, alone.variance,
                                                            alone.error)


def test_run_request_lowers_the_energy():
    from qmctorch_gb300.serving import Request, hydrogen_chain, single_point
    r = Request(atoms=hydrogen_chain(4, 1.0), nwalkers=4096, nstep=200, seed=3, kind="run",
                nepoch=20, lr=2e-2, nstep_update=25, precision="fp64")
    res = single_point(r)
    e = np.asarray(res.energies)
    assert np.all(np.isfinite(e)) and e[-5:].mean() < e[:5].mean()


def test_auto_precision_follows_the_probe():
    """precision="auto" (the default) runs the mixed method where its psi
    agrees with FP64 within 1e-4 (median over 256 seeded positions) and FP64
    elsewhere: a short chain samples in mixed precision, a long one (Slater
    matrices with condition numbers ~1e10) in FP64; each result records the
    method and the probe's error."""
    from qmctorch_gb300.serving import AUTO_PSI_TOL, Request, VMCServer, hydrogen_chain
    srv = VMCServer(nstreams=2)
    srv.submit(Request(atoms=hydrogen_chain(4, 0.95), nwalkers=512, nstep=20, seed=1))
    srv.submit(Request(atoms=hydrogen_chain(24, 0.95), nwalkers=512, nstep=20, seed=2))
    res = sorted(srv.run(), key=lambda r: r.rid)
    assert [r.precision for r in res] == ["mixed", "fp64"]
    assert res[0].mixed_psi_err <= AUTO_PSI_TOL < res[1].mixed_psi_err
    assert all(np.isfinite(r.energy) for r in res)
