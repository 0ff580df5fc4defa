"""Benchmark of the VMC hot path on GB300.

Workload (the reference config the headline metric is quoted on): H2O,
cc-pVDZ basis (25 cartesian AOs, 10 electrons), SlaterJastrow with
single_double(4,4) determinants (27 configurations) and the Pade e-e
Jastrow, 16384 walkers, Metropolis all-electron Gaussian moves with step 0.2.

One bench step = one persistent Metropolis launch advancing every walker by
``--mc-steps`` all-electron moves (walker-steps = walkers x moves). The
local-energy throughput (E_L/s) of the fused local-energy kernel on the same
walkers is measured beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0). With N > 1 (torchrun) every rank runs an
independent replica of the workload on its own GPU (walkers are independent
Markov chains; no collective on the data path) and the value is the sum over
ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

H2O = "O 0 0 0.1173; H 0 0.7572 -0.4692; H 0 -0.7572 -0.4692"
CONFIGS = "single_double(4,4)"
STEP_SIZE = 0.2
L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2
NWALKERS = 16384
# DRAM bytes (read + write) of one metropolis_kernel<float> launch on this workload, from
# ncu (profiles/metropolis_mixed_h2o_ccpvdz_16384w.md); independent of the step count
TRAFFIC_PER_LAUNCH = 4.55e6
C6H6 = ("C 1.39 0 0; C 0.695 1.20377 0; C -0.695 1.20377 0; C -1.39 0 0; "
        "C -0.695 -1.20377 0; C 0.695 -1.20377 0; H 2.48 0 0; H 1.24 2.14774 0; "
        "H -1.24 2.14774 0; H -2.48 0 0; H -1.24 -2.14774 0; H 1.24 -2.14774 0")
METRIC = ("walker-steps/s (Metropolis all-electron, mixed-precision method; "
          "E_L/s and the plain FP64 method alongside)")


def workload_config(args, nw):
    return {"workload": "h2o_ccpvdz_single_double44_16384w",
            "molecule": "H2O cc-pVDZ (25 cart AOs, 10 e)", "configs": CONFIGS,
            "nwalkers_per_gpu": nw, "mc_steps_per_step": args.mc_steps, "step_size": STEP_SIZE,
            "method": "mixed (FP32 + FP64 refinement)",
            "l2": "flushed between timed steps (256 MB write)"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=8)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--nwalkers", type=int, default=16384)
    p.add_argument("--c6h6-walkers", type=int, default=65536)
    p.add_argument("--serve-requests", type=int, default=48)
    p.add_argument("--serve-rates", type=float, nargs="*", default=[10.0, 40.0, 160.0])
    p.add_argument("--serve-budget-gb", type=int, default=32)
    p.add_argument("--skip", default="",
                   help="comma list of sections to leave out (c6h6, serving, small, modules, "
                        "mo_tc, h_n, precision, drift, hmc, e2e); for short profiling runs")
    p.add_argument("--c6h6-sweeps", type=int, default=4,
                   help="all-elec-iter sweeps per timed C6H6 launch (mixed method)")
    p.add_argument("--mc-steps", type=int, default=100)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--kernels", action="store_true",
                   help="time every kernel of the path once per precision on the workload "
                        "(psi, local energy, pooling, potentials, gradients, adjoints) and exit: "
                        "the launch list of the per-kernel profiles")
    return p.parse_args()


def seeded_positions(mol, nw, seed):
    """Electrons placed on their atoms, offset by N(0, 1 bohr^2) per coordinate."""
    rng = np.random.default_rng(seed)
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)[: mol.nelec]
    return (centers[None] + rng.normal(size=(nw, mol.nelec, 3))).reshape(nw, -1)


# ----------------------------------------------------------------------------
# CPU side: the oracle (the reference algorithm restated in numpy)
# ----------------------------------------------------------------------------
def _cpu_worker(args):
    nw, nstep, seed = args
    import os as _os
    _os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle import qmc_oracle as orc
    from qmctorch_gb300.scf import Molecule
    # the Hueckel orbitals: the oracle's arithmetic does not depend on the MO
    # values, and the SCF of each worker would fall inside the timed wall
    mol = Molecule(H2O, unit="angs", basis="cc-pvdz", calculator="huckel")
    rng = np.random.default_rng(seed)
    fc = np.random.default_rng(7).uniform(size=27)
    wf = orc.OracleSlaterJastrow(mol, configs=CONFIGS, fc_weight=fc)
    pos = seeded_positions(mol, nw, seed)
    sig = orc.metropolis_sigma(STEP_SIZE)
    props = rng.normal(size=(nstep, nw, 3 * mol.nelec)) * sig
    unif = rng.uniform(size=(nstep, nw))
    t0 = time.perf_counter()
    orc.metropolis_replay(wf.pdf, pos, props, unif, ntherm=nstep - 1)
    return time.perf_counter() - t0, nw * nstep


def cpu_baseline(target_seconds, steps=1, warmup=0):
    """Oracle Metropolis on the host cores: one spawn process per core, each
    advancing its own bounded walker sample. ``steps`` timed rounds (after
    ``warmup`` untimed ones) of about ``target_seconds`` each; returns
    walker-steps/s over the timed wall time and the wall time per round."""
    ncores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    nstep = 2
    total, walls = 0, []
    with ctx.Pool(ncores) as pool:
        # calibrate: one small chunk per core, all cores busy
        res = pool.map(_cpu_worker, [(64, 2, k) for k in range(ncores)])
        rate1 = min(n / dt for dt, n in res)
        nw = max(16, int(rate1 * target_seconds / 1.1) // nstep)
        for i in range(warmup + steps):
            t0 = time.perf_counter()
            res = pool.map(_cpu_worker, [(nw, nstep, 100 + 37 * i + k) for k in range(ncores)])
            if i >= warmup:
                walls.append(time.perf_counter() - t0)
                total += sum(r[1] for r in res)
    wall = sum(walls)
    return {"value": total / wall, "unit": "walker-steps/s", "cores": ncores, "kind": "port",
            "ms_per_round": wall * 1e3 / len(walls),
            "sample": "%d round(s) of %d processes x %d walkers x %d all-electron steps "
                      "(H2O cc-pVDZ single_double(4,4), numpy oracle), %.1f s wall timed"
                      % (len(walls), ncores, nw, nstep, wall)}


# ----------------------------------------------------------------------------
# GPU side
# ----------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        outdir = os.environ.get("QMC_BENCH_OUT", os.path.join(ROOT, "bench_out"))
        self.path = os.path.join(outdir, "clocks_rank%d.csv" % index)

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def probe_peaks(torch, lib, device):
    """FP64 / FP32 FMA and exp throughput of this GPU (kernels of the library)."""
    import ctypes
    nsm = torch.cuda.get_device_properties(device).multi_processor_count
    blocks = nsm * 8
    out = torch.empty(blocks * 256, dtype=torch.float64, device=device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    res = {}
    for kind, name, iters, per in ((0, "fp64_gflops", 2000, 16), (1, "fp32_gflops", 20000, 16),
                                   (2, "fp32_exp_gps", 10000, 8), (3, "fp64_exp_gps", 100, 8),
                                   (4, "fp64_exp_table_gps", 100, 8)):
        lib.qmc_probe_fma(kind, blocks, iters, ctypes.c_void_p(out.data_ptr()), stream)
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            lib.qmc_probe_fma(kind, blocks, iters, ctypes.c_void_p(out.data_ptr()), stream)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = max(best, per * iters * blocks * 256 / (ms * 1e-3) / 1e9)
        res[name] = best
    return res


def count_fp64_flops_per_psi(wf):
    """Algorithmic FP64 work of one psi evaluation in the kernel, counted from
    the wave-function tables (flop = one add, multiply or FMA-half; an exp
    counts as one evaluation, listed separately):
      AO->MO contraction 2*Ne*Nao*Nmo_u (the reference's GEMM figure),
      radial sums 2*Ne*(weights) + polynomial 3*Ne*Nao,
      e-e pairs 12 flop + 1 sqrt + 1 division each,
      LU 2/3 n^3 + solves 2 n^2 (Nmo_u - n) per spin, CI sum 3*ncfg."""
    bt = wf.ao._tables
    ne, nao, nmu = wf.nelec, wf.mo.mo_scf.shape[0], wf.highest_occ_mo
    flops = 2 * ne * nao * nmu + 2 * ne * bt.nweight + 3 * ne * nao + 6 * ne * bt.ngroup
    npair = ne * (ne - 1) // 2
    flops += 12 * npair
    for n in (wf.mol.nup, wf.mol.ndown):
        flops += int(2 * n ** 3 / 3) + 2 * n * n * (nmu - n)
    flops += 3 * wf.nci
    exps = ne * bt.ngprim + 1
    return flops, exps


def _timed(torch, fn, steps, flush):
    """CUDA-event time (s) of `steps` calls of fn(i) on the current stream,
    L2 flushed (outside the events) before each call."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for i in range(steps):
        flush.fill_(float(i))
        ev[i][0].record()
        fn(i)
        ev[i][1].record()
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / 1e3


def precision_study(torch, wf64, wfm, x_eq, sampler, nfixed=100_000):
    """Per-walker psi / E_L error of the mixed method against the FP64 method
    on `nfixed` fixed positions (snapshots of an equilibrated FP64 chain)."""
    snaps, n = [], 0
    x = x_eq.clone()
    while n < nfixed:
        sampler.advance(wf64.pdf, x, nstep=10)
        snaps.append(x.clone())
        n += x.shape[0]
    X = torch.cat(snaps)[:nfixed]
    with torch.no_grad():
        e64 = wf64.local_energy(X).reshape(-1).double()
        em = wfm.local_energy(X).reshape(-1).double()
        p64 = wf64(X).reshape(-1).double()
        pm = wfm(X).reshape(-1).double()
    de = (em - e64).abs()
    dp = ((pm - p64) / p64).abs()
    return {"n_positions": int(nfixed),
            "mean_eloc_fp64": float(e64.mean()), "mean_eloc_mixed": float(em.mean()),
            "mean_eloc_diff_ha": float(em.mean() - e64.mean()),
            "eloc_abs_err_median_ha": float(de.median()), "eloc_abs_err_p99_ha": float(torch.quantile(de.float(), 0.99)),
            "eloc_abs_err_max_ha": float(de.max()),
            "psi_rel_err_median": float(dp.median()), "psi_rel_err_max": float(dp.max()),
            "stat_error_of_mean_ha": float(e64.std() / nfixed ** 0.5)}


def metropolis_capi(torch, lib, wf, x, nstep, move_type, step, seed, generic=False, scratch=None):
    """qmc_metropolis_run on x (advanced in place) on the current stream;
    generic=True requests psi_out, which selects the kernel that re-evaluates
    psi for every move instead of the Sherman-Morrison sampler."""
    import ctypes

    from qmctorch_gb300 import _lib
    nw = x.shape[0]
    call = wf._desc(x.device)
    need = lib.qmc_metropolis_scratch_bytes(call.ref, nw)
    if scratch is None or scratch.numel() < need:
        scratch = torch.empty(max(need, 1), dtype=torch.uint8, device=x.device)
    psi = torch.empty(nw, dtype=torch.float64, device=x.device) if generic else None
    a = _lib.MetropolisArgs()
    a.pos = ctypes.c_void_p(x.data_ptr())
    a.nwalkers, a.nstep, a.ntherm, a.ndecor = nw, nstep, nstep, 1
    a.move_type, a.proba, a.step_size, a.seed, a.step_offset = move_type, 0, step, seed, 0
    a.psi_out = ctypes.c_void_p(psi.data_ptr()) if generic else None
    _lib.check(lib.qmc_metropolis_run(call.ref, a, ctypes.c_void_p(scratch.data_ptr()),
                                      scratch.numel(),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "qmc_metropolis_run")
    return scratch, psi


def bench_h_n(torch, lib, device, flush, nw=16384, nstep=50):
    """Walker-steps/s of the mixed-method Metropolis kernel (all-electron moves,
    step 0.2) on the serving workload's molecules: linear H_n sto-3g chains,
    n = 2, 4, ..., 32 at 0.95 A spacing, single determinant + Pade e-e Jastrow,
    16384 walkers, one launch of 50 steps per timed call."""
    from qmctorch_gb300.scf import Molecule
    from qmctorch_gb300.serving import hydrogen_chain
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    out = {"workload": "h_n_sto3g_ground_state_%dw_%d_steps" % (nw, nstep), "walker_steps_per_s": {}}
    for n in range(2, 33, 2):
        mol = Molecule(hydrogen_chain(n, 0.95), unit="angs", basis="sto-3g")
        wf = SlaterJastrow(mol, cuda=True, precision="mixed")
        x = torch.as_tensor(seeded_positions(mol, nw, seed=n), device=device)
        scr, _ = metropolis_capi(torch, lib, wf, x, nstep, 0, STEP_SIZE, 5)
        torch.cuda.synchronize()
        t = _timed(torch, lambda i: metropolis_capi(torch, lib, wf, x, nstep, 0, STEP_SIZE, 6 + i,
                                                    scratch=scr), 3, flush) / 3
        out["walker_steps_per_s"]["H%d" % n] = nw * nstep / t
        # stated error of the mixed method: psi against the FP64 method on 4096 of
        # the sampled positions (FP32 MO values: about kappa * 6e-8 relative)
        wf64 = SlaterJastrow(mol, cuda=True, precision="fp64")
        with torch.no_grad():
            xs = x[:4096].clone()
            p64 = wf64(xs).reshape(-1)
            rel = ((wf(xs).reshape(-1) - p64) / p64).abs()
        out.setdefault("psi_rel_err_vs_fp64_median", {})["H%d" % n] = float(rel.median())
        out.setdefault("psi_rel_err_vs_fp64_p90", {})["H%d" % n] = float(torch.quantile(rel, 0.9))
        if n % 8 == 0:  # the plain method on the chains the serving stream sends to it
            x64 = x.clone()
            scr64, _ = metropolis_capi(torch, lib, wf64, x64, 10, 0, STEP_SIZE, 5)
            torch.cuda.synchronize()
            t64 = _timed(torch, lambda i: metropolis_capi(torch, lib, wf64, x64, 10, 0, STEP_SIZE,
                                                          6 + i, scratch=scr64), 2, flush) / 2
            out.setdefault("fp64_walker_steps_per_s", {})["H%d" % n] = nw * 10 / t64
    return out


def bench_c6h6(torch, lib, args, device, flush, rank):
    """C6H6 cc-pVDZ, single determinant + Pade e-e Jastrow, all-elec-iter
    sweeps (42 single-electron moves each) with step 0.1: walker-sweeps/s of
    the Sherman-Morrison sampler in both methods, E_L/s, and the kernel that
    re-evaluates psi for every move on a 4096-walker subset."""
    import ctypes

    from qmctorch_gb300 import _lib
    from qmctorch_gb300.scf import Molecule
    from qmctorch_gb300.wavefunction import SlaterJastrow
    mol = Molecule(C6H6, unit="angs", basis="cc-pvdz")
    nw = args.c6h6_walkers
    x0 = torch.as_tensor(seeded_positions(mol, nw, seed=50 + rank), device=device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = {"workload": "c6h6_ccpvdz_ground_state_%dw_all_elec_iter" % nw,
           "molecule": "C6H6 cc-pVDZ (120 cart AOs, 42 e)", "configs": "ground_state",
           "move": "all-elec-iter (one sweep = 42 single-electron moves)", "step_size": 0.1,
           "nwalkers": nw}
    wfs = {}
    for name in ("mixed", "fp64"):
        wf = SlaterJastrow(mol, configs="ground_state", cuda=True, precision=name)
        wfs[name] = wf
        x = x0.clone()
        sweeps = args.c6h6_sweeps if name == "mixed" else 1
        steps = args.steps if name == "mixed" else max(2, args.steps // 4)
        scr, _ = metropolis_capi(torch, lib, wf, x, 1, 2, 0.1, 11)
        for _ in range(max(1, args.warmup if name == "mixed" else 1)):
            metropolis_capi(torch, lib, wf, x, sweeps, 2, 0.1, 12, scratch=scr)
        torch.cuda.synchronize()
        t = _timed(torch, lambda i: metropolis_capi(torch, lib, wf, x, sweeps, 2, 0.1, 100 + i,
                                                     scratch=scr), steps, flush)
        call = wf._desc(device)
        el_scr = torch.empty(lib.qmc_scratch_bytes(call.ref, nw, 1), dtype=torch.uint8,
                             device=device)
        eloc = torch.empty(nw, dtype=torch.float64, device=device)

        def el_call(i):
            _lib.check(lib.qmc_wf_local_energy(call.ref, ctypes.c_void_p(x.data_ptr()), nw,
                                               ctypes.c_void_p(eloc.data_ptr()), None, None,
                                               ctypes.c_void_p(el_scr.data_ptr()),
                                               el_scr.numel(), stream), "qmc_wf_local_energy")
        el_call(0)
        torch.cuda.synchronize()
        el_t = _timed(torch, el_call, 3, flush)
        # the kernel that re-evaluates psi for every move, on a subset
        ng = 4096
        xg = x[:ng].clone()
        gscr, _ = metropolis_capi(torch, lib, wf, xg, 1, 2, 0.1, 13, generic=True)
        torch.cuda.synchronize()
        g_t = _timed(torch, lambda i: metropolis_capi(torch, lib, wf, xg, 1, 2, 0.1, 200 + i,
                                                       generic=True, scratch=gscr), 2, flush)
        out[name] = {"walker_sweeps_per_s": nw * sweeps * steps / t,
                     "ms_per_sweep": t * 1e3 / (sweeps * steps), "timed_launches": steps,
                     "sweeps_per_launch": sweeps, "el_per_s": nw * 3 / el_t,
                     "reevaluating_kernel_walker_sweeps_per_s": ng * 2 / g_t}
        out[name]["speedup_vs_reevaluating_kernel"] = (
            out[name]["walker_sweeps_per_s"] / out[name]["reevaluating_kernel_walker_sweeps_per_s"])
    out["speedup_mixed_vs_fp64"] = {
        "walker_sweeps": out["mixed"]["walker_sweeps_per_s"] / out["fp64"]["walker_sweeps_per_s"],
        "el": out["mixed"]["el_per_s"] / out["fp64"]["el_per_s"]}
    # precision of the mixed method on the positions the chains reached
    with torch.no_grad():
        e64 = wfs["fp64"].local_energy(x).reshape(-1)
        em = wfs["mixed"].local_energy(x).reshape(-1)
        de = (em - e64).abs()
        out["precision_vs_fp64"] = {
            "n_positions": int(x.shape[0]),
            "mean_eloc_fp64": float(e64.mean()), "mean_eloc_mixed": float(em.mean()),
            "mean_eloc_diff_ha": float((em - e64).mean()),
            "eloc_abs_err_median_ha": float(de.median()),
            "eloc_abs_err_p99_ha": float(torch.quantile(de[:min(len(de), 1 << 20)], 0.99)),
            "stat_error_of_mean_ha": float(e64.std() / len(e64) ** 0.5)}
    return out


def bench_h2_lih(torch, device):
    """The reference's small configurations through the public API (plain
    FP64 method): H2 sto-3g Solver.single_point (4096 walkers, 500 steps,
    200 burn-in, every later step kept: 1.23 M samples) and LiH sto-3g
    cas(2,2) Solver.run (8192 walkers, 50 epochs, Adam lr 1e-3, manual
    gradient through the hand-written adjoint, 25-step resampling)."""
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.scf import Molecule
    from qmctorch_gb300.solver import Solver
    from qmctorch_gb300.wavefunction import SlaterJastrow
    out = {}
    mol = Molecule("H 0 0 -0.37; H 0 0 0.37", unit="angs", basis="sto-3g")
    wf = SlaterJastrow(mol, configs="ground_state", cuda=True, precision="fp64")
    smp = Metropolis(nwalkers=4096, nstep=500, step_size=0.2, ntherm=200, ndecor=1, nelec=2,
                     init=mol.domain("atomic"), cuda=True, seed=5)
    solver = Solver(wf=wf, sampler=smp)
    solver.single_point(with_tqdm=False)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    obs = solver.single_point(with_tqdm=False)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    out["h2_single_point"] = {
        "workload": "h2_sto3g_4096w_500steps_single_point", "wall_s": dt,
        "walker_steps_per_s": 4096 * 500 / dt, "samples": int(obs.local_energy.numel()),
        "energy": float(obs.energy), "error": float(obs.error)}
    mol = Molecule("Li 0 0 0; H 0 0 1.595", unit="angs", basis="sto-3g")
    wf = SlaterJastrow(mol, configs="cas(2,2)", cuda=True, precision="fp64")
    smp = Metropolis(nwalkers=8192, nstep=200, step_size=0.2, nelec=mol.nelec,
                     init=mol.domain("atomic"), cuda=True, seed=6)
    opt = torch.optim.Adam(wf.parameters(), lr=1e-3)
    solver = Solver(wf=wf, sampler=smp, optimizer=opt)
    solver.run(2)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    obs = solver.run(50)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    e = [float(v) for v in obs.energy]
    out["lih_run"] = {"workload": "lih_sto3g_cas22_8192w_50_epochs", "wall_s": dt,
                      "epochs_per_s": 50 / dt, "energy_first": e[0], "energy_last": e[-1]}
    return out


def bench_drift(torch, wf, x_eq, nstep_kernel=50, nstep_loop=5):
    """Drift-diffusion sampler (GeneralizedMetropolis) on H2O cc-pVDZ
    single_double(4,4), FP64, the walkers of the headline: one qmc_drift_run
    launch per call (device generator) against the host loop of one density
    and one gradient kernel call per step (the drift of the Jacobi gradient
    kernel), both through GeneralizedMetropolis.__call__ from device walkers."""
    from qmctorch_gb300.sampler import GeneralizedMetropolis

    class HostLoopPdf:  # wf.pdf under another name: the sampler's host loop
        def __init__(self, wf):
            self.__self__, self.__name__ = wf, "pdf_host_loop"

        def __call__(self, x, return_grad=False):
            return self.__self__.pdf(x, return_grad=return_grad)

    nw = x_eq.shape[0]
    out = {"workload": "h2o_ccpvdz_sd44_%dw_fp64" % nw}
    for name, pdf, nstep in (("kernel", wf.pdf, nstep_kernel),
                             ("host_loop", HostLoopPdf(wf), nstep_loop)):
        s = GeneralizedMetropolis(nwalkers=nw, nstep=nstep, step_size=0.05, ntherm=-1,
                                  nelec=wf.mol.nelec, ndim=3, cuda=True, seed=17)
        s(pdf, pos=x_eq.clone(), with_tqdm=False)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s(pdf, pos=x_eq.clone(), with_tqdm=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[name] = {"nstep": nstep, "wall_s": dt, "walker_steps_per_s": nw * nstep / dt,
                     "acceptance": s.last_acceptance}
    out["speedup"] = out["kernel"]["walker_steps_per_s"] / out["host_loop"]["walker_steps_per_s"]
    return out


def bench_hmc(torch, wf, x_eq, nstep_kernel=10, nstep_loop=2, traj=5):
    """HMC sampler (Hamiltonian) on H2O cc-pVDZ single_double(4,4), FP64, the
    walkers of the headline, trajectories of 5 leapfrog steps: one qmc_hmc_run
    launch per call (device generator) against the host loop of one density
    and one gradient kernel call per leapfrog point, both through
    Hamiltonian.__call__ from device walkers. Unit: walker-trajectories/s."""
    from qmctorch_gb300.sampler import Hamiltonian

    class HostLoopPdf:  # wf.pdf under another name: the sampler's host loop
        def __init__(self, wf):
            self.__self__, self.__name__ = wf, "pdf_host_loop"

        def __call__(self, x, return_grad=False):
            return self.__self__.pdf(x, return_grad=return_grad)

    nw = x_eq.shape[0]
    out = {"workload": "h2o_ccpvdz_sd44_%dw_fp64_L%d" % (nw, traj)}
    for name, pdf, nstep in (("kernel", wf.pdf, nstep_kernel),
                             ("host_loop", HostLoopPdf(wf), nstep_loop)):
        s = Hamiltonian(nwalkers=nw, nstep=nstep, step_size=0.02, L=traj, ntherm=-1,
                        nelec=wf.mol.nelec, ndim=3, cuda=True, seed=19)
        s(pdf, pos=x_eq.clone(), with_tqdm=False)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s(pdf, pos=x_eq.clone(), with_tqdm=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[name] = {"nstep": nstep, "wall_s": dt, "walker_trajectories_per_s": nw * nstep / dt,
                     "acceptance": s.last_acceptance}
    out["speedup"] = (out["kernel"]["walker_trajectories_per_s"]
                      / out["host_loop"]["walker_trajectories_per_s"])
    return out


def bench_staged(torch, wf, x, flush):
    """The module kernels a caller of a single layer gets (wf.ao, wf.mo,
    wf.jastrow; FP64, reference tensor layouts) on the bench walkers:
    time per call and achieved HBM bandwidth of the bytes they must move
    (positions in, the layer's output tensors out)."""
    peak = 6800.0
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f).get("hbm_gbs", peak))
    except Exception:
        pass
    nw, nc = x.shape
    ne = nc // 3
    out = {}
    with torch.no_grad():
        ao = wf.ao(x)
        nao = ao.shape[-1]
        nmo = wf.mo(ao).shape[-1]
        cases = {
            "ao_values": (lambda: wf.ao(x), nw * nc * 8 + nw * ne * nao * 8),
            "ao_values_grad_lap": (lambda: wf.ao(x, derivative=[0, 1, 2], sum_grad=False),
                                   nw * nc * 8 + nw * ne * nao * 8 * 5),
            "mo_from_ao": (lambda: wf.mo(ao), nw * ne * nao * 8 + nw * ne * nmo * 8),
            "jastrow_value_grad_lap": (lambda: wf.jastrow(x, derivative=[0, 1, 2], sum_grad=False),
                                       nw * nc * 8 + nw * 8 + nw * 3 * ne * 8 + nw * ne * 8),
        }
        for name, (fn, nbytes) in cases.items():
            fn()
            torch.cuda.synchronize()
            t = _timed(torch, lambda i: fn(), 5, flush) / 5
            out[name] = {"ms": t * 1e3, "algorithmic_bytes": nbytes,
                         "achieved_gbs": nbytes / t / 1e9, "frac_of_hbm": nbytes / t / 1e9 / peak}
    out["hbm_peak_gbs"] = peak
    return out


def bench_mo_tensor_core(torch, device, flush, nw_c6h6=16384, nw_h2o=16384):
    """AO->MO of the module path (wf.mo(ao)) on the tensor cores
    (qmc_mo_eval_tc, split-BF16 x3, FP32 accumulation) beside the FP64 kernel
    (qmc_mo_eval): C6H6 cc-pVDZ (120 AOs -> 114 MOs) and H2O cc-pVDZ
    (25 -> 24) at seeded positions, L2 flushed between timed calls. Reports
    time per call, algorithmic HBM bytes (AO read + MO written, FP64) per
    second against the copy peak, the BF16 tensor work the MMAs execute
    (3 split products over the padded 128-row tiles) against the BF16 peak,
    and the largest error relative to |AO| @ |W|."""
    from qmctorch_gb300.scf import Molecule
    from qmctorch_gb300.wavefunction import SlaterJastrow
    peaks = {"hbm_gbs": 6800.0, "bf16_tflops": 1917.0}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks.update({k: float(v) for k, v in json.load(f).items() if k in peaks})
    except Exception:
        pass
    out = {"hbm_peak_gbs": peaks["hbm_gbs"], "bf16_peak_tflops": peaks["bf16_tflops"]}
    for tag, geom, nw in (("c6h6_ccpvdz", C6H6, nw_c6h6), ("h2o_ccpvdz", H2O, nw_h2o)):
        mol = Molecule(geom, unit="angs", basis="cc-pvdz")
        wf64 = SlaterJastrow(mol, cuda=True, precision="fp64")
        wfm = SlaterJastrow(mol, cuda=True, precision="mixed")
        x = torch.as_tensor(seeded_positions(mol, nw, seed=11), device=device)
        with torch.no_grad():
            ao = wf64.ao(x)
            rows, nao = nw * mol.nelec, ao.shape[-1]
            ref = wf64.mo(ao)
            got = wfm.mo(ao)
            nmo = ref.shape[-1]
            W = (wf64.mo.mo_scf * wf64.mo.mo_modifier).to(torch.float64)
            scale = (ao.abs().reshape(rows, nao) @ W.abs()).reshape(ref.shape)
            err = float(((got - ref).abs() / (scale + 1e-300)).max())
            # the kernels through the C ABI (descriptor built, output allocated
            # once), and the module call wf.mo(ao) (with its status check)
            import ctypes

            from qmctorch_gb300 import _lib
            from qmctorch_gb300.wavefunction import runtime as rt
            lib = _lib.lib()
            xa = ao.reshape(-1, nao).contiguous()
            dst = torch.empty((rows, nmo), dtype=torch.float64, device=device)

            def capi(wf, fn):
                call = rt.build_desc(device, wf.ao, mo=wf.mo)
                f = getattr(lib, fn)
                sh = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
                return lambda i: f(call.ref, ctypes.c_void_p(xa.data_ptr()), rows,
                                   ctypes.c_void_p(dst.data_ptr()), sh)

            t_tc = _timed(torch, capi(wfm, "qmc_mo_eval_tc"), 5, flush) / 5
            _lib.check(lib.qmc_mo_eval_tc_status(None), "qmc_mo_eval_tc")
            t_64 = _timed(torch, capi(wf64, "qmc_mo_eval"), 3, flush) / 3
            t_mod = _timed(torch, lambda i: wfm.mo(ao), 5, flush) / 5
        nbytes = rows * (nao + nmo) * 8
        kp, npad = (nao + 15) // 16 * 16, (nmo + 15) // 16 * 16
        tc_flops = 2.0 * ((rows + 127) // 128 * 128) * npad * 3 * kp
        out[tag] = {"rows": rows, "nao": nao, "nmo": nmo, "ms_tc": t_tc * 1e3,
                    "ms_fp64": t_64 * 1e3, "speedup_vs_fp64": t_64 / t_tc,
                    "ms_tc_module_call": t_mod * 1e3,
                    "algorithmic_bytes": nbytes, "achieved_gbs": nbytes / t_tc / 1e9,
                    "frac_of_hbm": nbytes / t_tc / 1e9 / peaks["hbm_gbs"],
                    "tensor_tflops": tc_flops / t_tc / 1e12,
                    "frac_of_bf16": tc_flops / t_tc / 1e12 / peaks["bf16_tflops"],
                    "max_err_rel_to_abs_product": err}
        del ao, ref, got, scale
    return out


def bench_serving(args):
    """Continuous-batching single-point server on a seeded Poisson stream of
    H_n sto-3g requests (n even in 2..32, spacing 0.7-1.2 A, walkers
    log-uniform 1024-16384, 100-1000 steps, mixed method), at each arrival rate
    of --serve-rates: p50 / p99 latency (arrival to result) and walker-steps/s
    over the makespan."""
    from qmctorch_gb300.serving import (VMCServer, latency_percentiles, poisson_stream,
                                        replay_stream)
    out = {"workload": "h_n_sto3g_single_point_stream", "requests_per_rate": args.serve_requests,
           "hbm_budget_bytes": args.serve_budget_gb << 30, "slice_steps": 256,
           "precision": "auto: the mixed method where its median psi error against FP64 "
                        "(256 seeded positions per molecule) is <= 1e-4, else FP64",
           "rates": []}
    # warm-up: build and load every shape once (kernels, plans, molecules)
    warm = VMCServer(hbm_budget=args.serve_budget_gb << 30)
    replay_stream(warm, poisson_stream(8, 1000.0, seed=99, smin=20, smax=20, wmin=256,
                                       wmax=256))
    for rate in args.serve_rates:
        srv = VMCServer(hbm_budget=args.serve_budget_gb << 30)
        stream = poisson_stream(args.serve_requests, rate, seed=0)
        res, makespan = replay_stream(srv, stream)
        ws = sum(r.nwalkers * r.nstep for r in res)
        lat = latency_percentiles(res)
        out["rates"].append({"lambda_per_s": rate, "completed": len(res),
                             "p50_latency_s": lat["p50"], "p99_latency_s": lat["p99"],
                             "walker_steps_per_s": ws / makespan, "makespan_s": makespan,
                             "launches": srv.launches,
                             "jobs_per_launch": srv.launched_jobs / max(srv.launches, 1),
                             "fp64_requests": sum(r.precision == "fp64" for r in res)})
    return out


def _r(v, k=4):
    return None if v is None else float("%.*g" % (k, v))


def summarize(line, results, args, units, world, m_met, m_el, f_met, f_el):
    """Compact record of the numbers beside the headline: the plain FP64
    method, E_L/s, the mixed-method error on fixed positions, the C6H6,
    serving, H_n and module-kernel figures."""
    nw = line["config"]["nwalkers_per_gpu"]
    out = {"fp64_walker_steps_per_s": _r(units * world / f_met),
           "mixed_over_fp64_walker_steps": _r(f_met / m_met),
           "el_per_s_mixed": _r(nw * args.steps * world / m_el),
           "el_per_s_fp64": _r(nw * args.steps * world / f_el),
           "mixed_over_fp64_el": _r(f_el / m_el),
           "acceptance": _r(results["mixed"]["accept"], 3)}
    p = line.get("precision_vs_fp64")
    if p:
        out["precision_1e5_positions"] = {"mean_eloc_diff_ha": _r(p["mean_eloc_diff_ha"], 3),
                                          "eloc_err_p99_ha": _r(p["eloc_abs_err_p99_ha"], 3),
                                          "psi_rel_err_median": _r(p["psi_rel_err_median"], 3)}
    c = line.get("c6h6_single_electron")
    if c:
        out["c6h6_walker_sweeps_per_s"] = {"mixed": _r(c["mixed"]["walker_sweeps_per_s"]),
                                           "fp64": _r(c["fp64"]["walker_sweeps_per_s"])}
        out["c6h6_el_per_s"] = {"mixed": _r(c["mixed"]["el_per_s"]),
                                "fp64": _r(c["fp64"]["el_per_s"])}
    sv = line.get("serving")
    if sv:
        out["serving"] = [{"lambda": r["lambda_per_s"], "p50_s": _r(r["p50_latency_s"], 3),
                           "p99_s": _r(r["p99_latency_s"], 3),
                           "ws_per_s": _r(r["walker_steps_per_s"], 3),
                           "jobs_per_launch": _r(r["jobs_per_launch"], 3)} for r in sv["rates"]]
    h = line.get("h_n_metropolis")
    if h:
        ws = h["walker_steps_per_s"]
        out["h_n_walker_steps_per_s"] = {k: _r(ws[k], 3) for k in ("H8", "H16", "H20", "H32")
                                         if k in ws}
        er = h.get("psi_rel_err_vs_fp64_median", {})
        out["h_n_mixed_psi_rel_err_median"] = {k: _r(er[k], 2) for k in ("H8", "H12", "H16", "H20")
                                               if k in er}
    mt = line.get("mo_tensor_core")
    if mt and "c6h6_ccpvdz" in mt:
        out["mo_tc_c6h6"] = {"ms": _r(mt["c6h6_ccpvdz"]["ms_tc"], 3),
                             "frac_of_hbm": _r(mt["c6h6_ccpvdz"]["frac_of_hbm"], 3)}
    sm = line.get("small_configs")
    if sm:
        out["h2_single_point_s"] = _r(sm["h2_single_point"]["wall_s"], 3)
        out["lih_epochs_per_s"] = _r(sm["lih_run"]["epochs_per_s"], 3)
    return out


def slowest_rank_times(torch, vals, device, world):
    """Per-quantity maximum of the ranks' timed durations (replicas: every
    rank runs its own walkers, the job takes as long as the slowest rank)."""
    loc = torch.tensor(vals, dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(loc, op=dist.ReduceOp.MAX)
    return loc.tolist()


def run_gb300(args):
    import ctypes

    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cpu = None
    if rank == 0:
        cpu = cpu_baseline(args.cpu_seconds)  # spawn pool before the first CUDA call
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=device)

    from qmctorch_gb300 import _lib
    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.scf import Molecule
    from qmctorch_gb300.wavefunction import SlaterJastrow

    torch.set_default_dtype(torch.float64)
    lib = _lib.lib()
    mol = Molecule(H2O, unit="angs", basis="cc-pvdz")
    wf64 = SlaterJastrow(mol, configs=CONFIGS, cuda=True, precision="fp64")
    fc = np.random.default_rng(7).uniform(size=wf64.nci)
    wf64.fc.weight.data = torch.as_tensor(fc, device=device).reshape(1, -1)
    wfm = SlaterJastrow(mol, configs=CONFIGS, cuda=True, precision="mixed")
    wfm.load_state_dict(wf64.state_dict())
    nw = args.nwalkers
    x0 = torch.as_tensor(seeded_positions(mol, nw, seed=rank), device=device)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    peaks = probe_peaks(torch, lib, device)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def sampler_for(seed):
        return Metropolis(nwalkers=nw, nstep=args.mc_steps, step_size=STEP_SIZE,
                          nelec=mol.nelec, init=mol.domain("atomic"), cuda=True, seed=seed)

    # equilibrate once with the FP64 chain; both methods start from these walkers
    eq = sampler_for(4321 + rank)
    x_eq = x0.clone()
    eq.advance(wf64.pdf, x_eq, nstep=500)
    barrier()

    results = {}
    clocks = ClockSampler(local)
    clocks.start()
    for name, wf in (("mixed", wfm), ("fp64", wf64)):
        x = x_eq.clone()
        s = sampler_for(1234 + rank)
        call = wf._desc(device)
        scr = torch.empty(lib.qmc_metropolis_scratch_bytes(call.ref, nw), dtype=torch.uint8,
                          device=device)
        acc = torch.zeros(nw, dtype=torch.int32, device=device)
        for _ in range(args.warmup):
            s.advance(wf.pdf, x, accepted=acc, scratch=scr)
        acc.zero_()
        barrier()
        met_s = _timed(torch, lambda i: s.advance(wf.pdf, x, accepted=acc, scratch=scr),
                       args.steps, flush)
        el_scr = torch.empty(lib.qmc_scratch_bytes(call.ref, nw, 1), dtype=torch.uint8,
                             device=device)
        eloc = torch.empty(nw, dtype=torch.float64, device=device)

        def el_call(i):
            _lib.check(lib.qmc_wf_local_energy(call.ref, ctypes.c_void_p(x.data_ptr()), nw,
                                               ctypes.c_void_p(eloc.data_ptr()), None, None,
                                               ctypes.c_void_p(el_scr.data_ptr()),
                                               el_scr.numel(), stream), "qmc_wf_local_energy")
        el_call(0)
        barrier()
        el_s = _timed(torch, el_call, args.steps, flush)
        results[name] = {"met_s": met_s, "el_s": el_s,
                         "accept": float(acc.sum()) / (nw * args.mc_steps * args.steps)}
    skip = set(filter(None, args.skip.split(",")))
    c6h6 = (bench_c6h6(torch, lib, args, device, flush, rank)
            if args.c6h6_walkers > 0 and "c6h6" not in skip else None)
    clk = clocks.stop()
    serving = (bench_serving(args) if (args.serve_requests > 0 and rank == 0
                                       and "serving" not in skip) else None)
    small = bench_h2_lih(torch, device) if rank == 0 and "small" not in skip else None
    staged = bench_staged(torch, wf64, x_eq, flush) if rank == 0 and "modules" not in skip else None
    drift = bench_drift(torch, wf64, x_eq) if rank == 0 and "drift" not in skip else None
    hmc = bench_hmc(torch, wf64, x_eq) if rank == 0 and "hmc" not in skip else None
    mo_tc = (bench_mo_tensor_core(torch, device, flush)
             if rank == 0 and "mo_tc" not in skip else None)
    h_n = bench_h_n(torch, lib, device, flush) if rank == 0 and "h_n" not in skip else None

    prec = (precision_study(torch, wf64, wfm, x_eq, sampler_for(777 + rank))
            if rank == 0 and "precision" not in skip else None)

    # --- end to end through the public API (mixed method), host buffers ---
    pos_host = x_eq.detach().cpu().pin_memory()
    s_e2e = Metropolis(nwalkers=nw, nstep=args.mc_steps, step_size=STEP_SIZE, nelec=mol.nelec,
                       init=mol.domain("atomic"), cuda=False, seed=99 + rank)
    out = s_e2e(wfm.pdf, pos=pos_host, with_tqdm=False)
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        out = s_e2e(wfm.pdf, pos=pos_host, with_tqdm=False)
    barrier()
    e2e_s = time.perf_counter() - t0
    h2d = pos_host.numel() * 8
    d2h = out.numel() * out.element_size() + pos_host.numel() * 8

    m_met, m_el, f_met, f_el, e2e_s = slowest_rank_times(
        torch, [results["mixed"]["met_s"], results["mixed"]["el_s"], results["fp64"]["met_s"],
                results["fp64"]["el_s"], e2e_s], device, world)
    units = nw * args.mc_steps * args.steps
    value = units * world / m_met
    if rank == 0:
        flops, exps = count_fp64_flops_per_psi(wf64)
        launch_units = nw * args.mc_steps
        ach_m = flops * launch_units / (m_met / args.steps) / 1e9
        ach_f = flops * launch_units / (f_met / args.steps) / 1e9
        hbm_alg = 2 * nw * 3 * mol.nelec * 8  # positions in and out, FP64
        hbm_peak = 6800.0
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                hbm_peak = float(json.load(f).get("hbm_gbs", hbm_peak))
        except Exception:
            pass
        fp32_peak = peaks["fp32_gflops"]
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "walker-steps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": m_met * 1e3 / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32+f64 (mixed)",
            "data": "synthetic (seeded walker positions; built-in cc-pVDZ tables, RHF MOs of this package's SCF)",
            "config": workload_config(args, nw),
            # compute roofline of the dominant kernel: counted flops per walker-step
            # (count_fp64_flops_per_psi: the work of one psi evaluation) x walker-steps
            # per launch / the launch's CUDA-event time, against the FP32 FMA rate
            # measured in this run; traffic = ncu DRAM bytes of one launch
            "roofline": {"bound": "fp32", "kernel": "metropolis_kernel_wide<float>",
                         "achieved": ach_m / 1e3, "peak": fp32_peak / 1e3, "unit": "TFLOP/s",
                         "frac": ach_m / fp32_peak, "traffic": TRAFFIC_PER_LAUNCH,
                         "flops_per_walker_step": flops,
                         "algorithmic_flops_per_launch": flops * launch_units,
                         "launch_ms": m_met * 1e3 / args.steps,
                         "peak_source": "FP32 FMA rate measured in this run (qmc_probe_fma; "
                                        "MEASURED_PEAKS.json holds no FP32 figure)"},
            "roofline_hbm": {"bound": "hbm", "kernel": "metropolis_kernel_wide<float>",
                             "achieved": hbm_alg / (m_met / args.steps) / 1e9,
                             "peak": hbm_peak, "unit": "GB/s",
                             "frac": hbm_alg / (m_met / args.steps) / 1e9 / hbm_peak,
                             "algorithmic_bytes_per_launch": hbm_alg,
                             "note": "positions in and out once per launch: not HBM-bound"},
            "roofline_fp64": {"bound": "fp64", "kernel": "metropolis_kernel<double>",
                              "achieved": ach_f, "peak": peaks["fp64_gflops"], "unit": "GFLOP/s",
                              "frac": ach_f / peaks["fp64_gflops"]},
            "peaks_measured": peaks,
            "cpu_baseline": cpu,
            "e2e": {"value": units * world / e2e_s, "unit": "walker-steps/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "api": "Metropolis.__call__(wf.pdf, pos=pinned host tensor) -> host samples "
                           "(mixed method)"},
            "c6h6_single_electron": c6h6,
            "serving": serving,
            "small_configs": small,
            "module_kernels": staged,
            "drift_sampler": drift,
            "hmc_sampler": hmc,
            "mo_tensor_core": mo_tc,
            "h_n_metropolis": h_n,
            "precision_vs_fp64": prec,
            "gpu_launches": 4 * args.steps,
            "clocks": clk,
        }
        # the headline's companions, last on the line so that a tail of the
        # output carries them
        line["summary"] = summarize(line, results, args, units, world, m_met, m_el, f_met, f_el)
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def run_kernels(args):
    """Each kernel of the path on the workload (H2O cc-pVDZ single_double(4,4),
    ``--nwalkers`` seeded positions after 200 FP64 Metropolis steps), both
    precisions: CUDA-event time per call (mean of 3 after one warm-up), one JSON
    line. The launch list a per-kernel ncu capture selects from."""
    import torch

    from qmctorch_gb300.sampler import Metropolis
    from qmctorch_gb300.scf import Molecule
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    device = torch.device("cuda", 0)
    mol = Molecule(H2O, unit="angs", basis="cc-pvdz")
    fc = np.random.default_rng(7).uniform(size=27)
    nw = args.nwalkers
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    out = {"workload": "h2o_ccpvdz_single_double44_%dw" % nw, "ms": {}}
    x = None
    for prec in ("mixed", "fp64"):
        wf = SlaterJastrow(mol, configs=CONFIGS, cuda=True, precision=prec)
        wf.fc.weight.data = torch.as_tensor(fc, device=device).reshape(1, -1)
        if x is None:
            x = torch.as_tensor(seeded_positions(mol, nw, seed=0), device=device)
            s = Metropolis(nwalkers=nw, nstep=200, step_size=STEP_SIZE, nelec=mol.nelec,
                           init=mol.domain("atomic"), cuda=True, seed=3)
            s.advance(wf.pdf if prec == "fp64" else SlaterJastrow(
                mol, configs=CONFIGS, cuda=True, precision="fp64").pdf, x)
        g = torch.as_tensor(np.random.default_rng(1).normal(size=nw), device=device)

        def psi_adj():
            for p_ in wf.parameters():
                p_.grad = None
            (wf(x).reshape(-1) * g).sum().backward()

        def el_adj():
            for p_ in wf.parameters():
                p_.grad = None
            (wf.local_energy(x).reshape(-1) * g).sum().backward()

        with torch.no_grad():
            mo = wf.mo(wf.ao(x))
        calls = {"psi": lambda: wf(x), "local_energy": lambda: wf.local_energy(x),
                 "pooling": lambda: wf.pool(mo), "potentials": lambda: wf._potentials(x),
                 "gradients": lambda: wf.gradients_jacobi(x), "psi_adjoint": psi_adj,
                 "local_energy_adjoint": el_adj}
        for name, fn in calls.items():
            if prec == "mixed" and name in ("pooling", "potentials", "gradients",
                                            "psi_adjoint", "local_energy_adjoint"):
                continue  # FP64 kernels whatever the method
            with torch.no_grad() if "adjoint" not in name else torch.enable_grad():
                fn()
                torch.cuda.synchronize()
                t = _timed(torch, lambda i: fn(), 3, flush) / 3
            out["ms"]["%s_%s" % (name, prec)] = t * 1e3
    print(json.dumps(out))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t0 = time.perf_counter()
    cpu = cpu_baseline(args.cpu_seconds / max(args.steps, 1), steps=args.steps,
                       warmup=args.warmup)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": cpu["value"], "unit": "walker-steps/s", "n_gpus": int(os.environ.get(
            "WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": cpu["ms_per_round"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded walker positions)",
        "config": workload_config(args, args.nwalkers),
        "cpu_baseline": cpu,
        "e2e": {"value": cpu["value"], "unit": "walker-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.kernels:
        run_kernels(a)
    else:
        run_gb300(a)
