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


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--nwalkers", type=int, default=16384)
    p.add_argument("--mc-steps", type=int, default=10)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
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
    mol = Molecule(H2O, unit="angs", basis="cc-pvdz")
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


def cpu_baseline(target_seconds, steps=1):
    """Oracle Metropolis on the host cores: one spawn process per core, each
    advancing its own bounded walker sample; returns walker-steps/s."""
    ncores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    # calibrate: one small chunk on one core
    with ctx.Pool(1) as pool:
        dt, n = pool.map(_cpu_worker, [(64, 2, 0)])[0]
    rate1 = n / dt
    per_core = max(32, int(rate1 * target_seconds / max(steps, 1) / 2))
    nstep = 2
    nw = max(16, per_core // nstep)
    results = []
    t0 = time.perf_counter()
    with ctx.Pool(ncores) as pool:
        for _ in range(steps):
            results += pool.map(_cpu_worker, [(nw, nstep, 100 + i) for i in range(ncores)])
    wall = time.perf_counter() - t0
    total = sum(r[1] for r in results)
    busy = max(r[0] for r in results) * steps
    return {"value": total / busy, "unit": "walker-steps/s", "cores": ncores, "kind": "port",
            "sample": "%d processes x %d walkers x %d all-electron steps (H2O cc-pVDZ "
                      "single_double(4,4), numpy oracle), %.1f s wall" % (ncores, nw, nstep, wall)}


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
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_rank%d.csv" % index)

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
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
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i]})
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
                                   (2, "fp32_exp_gps", 10000, 8), (3, "fp64_exp_gps", 500, 8)):
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


def run_gb300(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cpu = None
    if rank == 0 and world >= 1:
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
    wf = SlaterJastrow(mol, configs=CONFIGS, cuda=True)
    fc = np.random.default_rng(7).uniform(size=wf.nci)
    wf.fc.weight.data = torch.as_tensor(fc, device=device).reshape(1, -1)
    nw = args.nwalkers
    x = torch.as_tensor(seeded_positions(mol, nw, seed=rank), device=device)
    sampler = Metropolis(nwalkers=nw, nstep=args.mc_steps, step_size=STEP_SIZE, nelec=mol.nelec,
                         init=mol.domain("atomic"), cuda=True, seed=1234 + rank)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    call = wf._desc(device)
    scr = torch.empty(lib.qmc_metropolis_scratch_bytes(call.ref, nw), dtype=torch.uint8,
                      device=device)
    acc = torch.zeros(nw, dtype=torch.int32, device=device)
    peaks = probe_peaks(torch, lib, device)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # warm-up (also equilibrates the walkers)
    for _ in range(args.warmup):
        sampler.advance(wf.pdf, x, accepted=acc, scratch=scr)
    wf.local_energy(x)
    barrier()

    clocks = ClockSampler(local)
    clocks.start()
    # --- device-resident Metropolis: K timed launches, L2 flushed between ---
    acc.zero_()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(float(i))
        ev[i][0].record()
        sampler.advance(wf.pdf, x, accepted=acc, scratch=scr)
        ev[i][1].record()
    barrier()
    wall_met = time.perf_counter() - t0
    met_ms = [a.elapsed_time(b) for a, b in ev]
    # --- local energies of the same walkers ---
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    el_call = wf._desc(device)
    el_scr = torch.empty(lib.qmc_scratch_bytes(el_call.ref, nw, 1), dtype=torch.uint8,
                         device=device)
    eloc = torch.empty(nw, dtype=torch.float64, device=device)
    import ctypes
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    barrier()
    for i in range(args.steps):
        flush.fill_(float(i))
        ev2[i][0].record()
        _lib.check(lib.qmc_wf_local_energy(el_call.ref, ctypes.c_void_p(x.data_ptr()), nw,
                                           ctypes.c_void_p(eloc.data_ptr()), None, None,
                                           ctypes.c_void_p(el_scr.data_ptr()), el_scr.numel(),
                                           stream), "qmc_wf_local_energy")
        ev2[i][1].record()
    barrier()
    clk = clocks.stop()
    el_ms = [a.elapsed_time(b) for a, b in ev2]
    accept_rate = float(acc.sum()) / (nw * args.mc_steps * args.steps)

    # --- end to end through the public API, host buffers ---
    pos_host = x.detach().cpu().pin_memory()
    sampler_e2e = Metropolis(nwalkers=nw, nstep=args.mc_steps, step_size=STEP_SIZE,
                             nelec=mol.nelec, init=mol.domain("atomic"), cuda=False,
                             seed=99 + rank)
    out = sampler_e2e(wf.pdf, pos=pos_host, with_tqdm=False)  # warm
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        out = sampler_e2e(wf.pdf, pos=pos_host, with_tqdm=False)
    barrier()
    e2e_s = time.perf_counter() - t0
    h2d = pos_host.numel() * 8
    d2h = out.numel() * out.element_size() + pos_host.numel() * 8

    # --- aggregate over ranks ---
    met_s = sum(met_ms) / 1e3
    el_s = sum(el_ms) / 1e3
    loc = torch.tensor([met_s, el_s, e2e_s, wall_met], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(loc, op=dist.ReduceOp.MAX)
    met_s, el_s, e2e_s, wall_met = loc.tolist()
    wsteps = nw * args.mc_steps * args.steps * world
    value = wsteps / met_s
    if rank == 0:
        flops, exps = count_fp64_flops_per_psi(wf)
        per_launch_ms = met_s * 1e3 / args.steps
        launch_wsteps = nw * args.mc_steps
        achieved = flops * launch_wsteps / (per_launch_ms * 1e-3) / 1e9
        line = {
            "metric": "walker-steps/s (Metropolis all-electron; E_L/s alongside)",
            "value": value,
            "unit": "walker-steps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": met_s * 1e3 / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic (seeded walker positions; built-in cc-pVDZ tables, extended-Hueckel MOs)",
            "config": {"workload": "h2o_ccpvdz_single_double44_16384w",
                       "molecule": "H2O cc-pVDZ (25 cart AOs, 10 e)", "configs": CONFIGS,
                       "nwalkers_per_gpu": nw, "mc_steps_per_step": args.mc_steps,
                       "step_size": STEP_SIZE, "method": "plain FP64",
                       "l2": "flushed between timed steps (256 MB write)"},
            "el_per_s": nw * args.steps * world / el_s,
            "ms_per_eloc_batch": el_s * 1e3 / args.steps,
            "acceptance": accept_rate,
            "roofline": {"bound": "fp64", "kernel": "metropolis_kernel",
                         "achieved": achieved, "peak": peaks["fp64_gflops"], "unit": "GFLOP/s",
                         "frac": achieved / peaks["fp64_gflops"], "traffic": None,
                         "flops_per_walker_step": flops, "exp_per_walker_step": exps,
                         "peak_source": "in-run FP64 FMA probe (qmc_probe_fma); "
                                        "MEASURED_PEAKS.json holds no FP64 figure"},
            "peaks_measured": peaks,
            "cpu_baseline": cpu,
            "e2e": {"value": wsteps / e2e_s, "unit": "walker-steps/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "api": "Metropolis.__call__(wf.pdf, pos=pinned host tensor) -> host samples"},
            "gpu_launches": 2 * args.steps,
            "clocks": clk,
            "wall_s_metropolis": wall_met,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t0 = time.perf_counter()
    cpu = cpu_baseline(args.cpu_seconds / max(args.steps, 1), steps=args.steps + args.warmup)
    line = {
        "impl": "reference",
        "metric": "walker-steps/s (Metropolis all-electron; E_L/s alongside)",
        "value": cpu["value"], "unit": "walker-steps/s", "n_gpus": int(os.environ.get(
            "WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "h2o_ccpvdz_single_double44_16384w", "configs": CONFIGS,
                   "step_size": STEP_SIZE},
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
    else:
        run_gb300(a)
