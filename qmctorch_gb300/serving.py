"""Continuous-batching VMC server on one GPU: single-point and VMC-run jobs.

The reference has no serving layer; its units of work are
``Solver.single_point()`` (solver_base.py:316-387: sample the wave function
with Metropolis, evaluate the local energy on the kept walkers, report mean,
variance and sampling error) and ``Solver.run()`` (solver.py:186-350: energy
minimisation with the manual gradient, an optimizer step per epoch and
``nstep_update`` resampling steps after it). A request is one of these:

* ``kind="single_point"``: ``nstep`` all-electron Metropolis steps from
  seeded positions (the last positions kept, as with the sampler's default
  ``ntherm = -1``), then the local energy and its statistics;
* ``kind="run"``: the same initial sampling, then ``nepoch`` epochs of
  (manual gradient 2 <(E_L - <E_L>) dpsi / psi> through the hand-written psi
  adjoint, Adam step, ``nstep_update`` resampling steps), then the final
  single point; the result also holds the mean local energy of every epoch.

Scheduling (``Scheduler``):

* requests queue FIFO and are admitted while their device footprint
  (positions, Metropolis scratch, local-energy scratch and outputs) fits the
  HBM budget and an active slot is free; a request that does not fit waits
  at the head of the queue;
* every admitted job's walker state stays resident on the device until it
  retires;
* the sampling work is cut into slices of ``slice_steps`` steps. Each
  scheduler pass gathers the jobs whose previous slice has finished, groups
  them by launch class (precision and MO column class; molecules of any size
  share a launch, each block running its job's own plan) and issues
  one ``qmc_metropolis_run_batch`` launch per group of up to ``QMC_MAX_BATCH``
  jobs, on a pool of CUDA streams, so groups overlap on the device and a job
  admitted while others run joins the next launch of its group;
* a job whose steps are done gets its local energies and compensated
  statistics (``qmc_reduce_stats``) on its stream, and retires when they are
  ready, releasing its budget.

Each walker's random stream is keyed by (seed, walker, step) and every
kernel's per-walker arithmetic is independent of the launch it runs in, so a
request's result is bitwise the same alone and in any mix.

The executor (device work) is separate from the scheduler so that the
scheduling logic is testable without a GPU.
"""
from __future__ import annotations

import ctypes
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

MAX_BATCH = 32  # QMC_MAX_BATCH of qmc_metropolis_run_batch
AUTO_PSI_TOL = 1e-4  # "auto" precision: largest median relative psi error of the mixed method


@dataclass
class Request:
    """One VMC single point: ``atoms`` (``Molecule`` syntax), ``nwalkers``
    walkers, ``nstep`` all-electron Metropolis steps of ``step_size``.
    ``calculator``: the molecular orbitals (``Molecule``): the extended-Hueckel
    guess by default -- an SCF per request on the scheduler's host thread
    would hold every other request while it runs -- or "pyscf" for this
    package's RHF."""
    atoms: str
    nwalkers: int
    nstep: int
    unit: str = "angs"
    basis: str = "sto-3g"
    calculator: str = "huckel"
    configs: str = "ground_state"
    step_size: float = 0.2
    seed: int = 0
    precision: str = "auto"      # "mixed", "fp64", or "auto" (GPUExecutor.precision_of)
    kind: str = "single_point"   # or "run"
    nepoch: int = 0              # run: optimisation epochs
    lr: float = 1e-3             # run: Adam learning rate
    nstep_update: int = 25       # run: resampling steps after each epoch
    rid: int = -1
    arrival: float = 0.0


@dataclass
class Result:
    rid: int
    energy: float
    variance: float
    error: float
    nwalkers: int
    nstep: int
    arrival: float
    admitted: float
    done: float
    energies: list = None  # run: mean local energy of each epoch
    precision: str = None  # the method that ran
    mixed_psi_err: float = None  # "auto": median relative psi error of the mixed method

    @property
    def latency(self):
        return self.done - self.arrival


@dataclass
class _Job:
    req: Request
    key: tuple
    footprint: int
    admitted: float
    steps_done: int = 0
    inflight: object = None      # token of the slice, gradient or energy work in flight
    phase: str = "sampling"      # sampling [-> grad -> sampling]* -> energy -> (retired)
    handle: object = None        # executor state
    order: int = 0
    target: int = 0              # Metropolis steps to reach before the next phase
    epoch: int = 0               # run: epochs done


class Scheduler:
    """FIFO admission under an HBM budget, slice-wise batched sampling,
    energy evaluation and retirement. ``executor`` provides the device work."""

    def __init__(self, executor, hbm_budget, max_active=256, slice_steps=64, nstreams=4,
                 clock=time.perf_counter):
        self.ex = executor
        self.budget = int(hbm_budget)
        self.max_active = max_active
        self.slice_steps = slice_steps
        self.nstreams = nstreams
        self.clock = clock
        self.queue = deque()
        self.active = []
        self.used = 0
        self.next_rid = 0
        self.results = {}
        self._stream_rr = 0
        self._order = 0
        self.launches = 0       # batched Metropolis launches
        self.launched_jobs = 0  # job slices in them

    # -- public API -------------------------------------------------------
    def submit(self, req):
        if req.kind not in ("single_point", "run"):
            raise ValueError("request kind must be 'single_point' or 'run'")
        req.rid = self.next_rid
        self.next_rid += 1
        req.arrival = self.clock()
        fp = self.ex.footprint(req)
        if fp > self.budget:
            raise ValueError("request %d needs %d bytes, more than the HBM budget %d"
                             % (req.rid, fp, self.budget))
        self.queue.append((req, fp))
        return req.rid

    def idle(self):
        return not self.queue and not self.active

    def poll(self):
        """One scheduler pass; returns the results retired in it."""
        done = self._retire()
        self._admit()
        self._launch()
        return done

    def run(self, sleep=2e-4):
        """Poll until every submitted request has a result."""
        out = []
        while not self.idle():
            got = self.poll()
            out += got
            if not got:
                time.sleep(sleep)
        return out

    # -- internals --------------------------------------------------------
    def _stream(self):
        s = self._stream_rr
        self._stream_rr = (self._stream_rr + 1) % self.nstreams
        return s

    def _retire(self):
        out = []
        keep = []
        for job in self.active:
            if job.inflight is not None and self.ex.ready(job.inflight):
                job.inflight = None
                if job.phase == "energy":
                    st = self.ex.stats(job.handle)
                    e, v, err, energies = st[:4]
                    r = Result(job.req.rid, e, v, err, job.req.nwalkers, job.req.nstep,
                               job.req.arrival, job.admitted, self.clock(), energies)
                    if len(st) > 4:  # the method that ran and, for "auto", its probe
                        r.precision, r.mixed_psi_err = st[4]
                    self.results[r.rid] = r
                    out.append(r)
                    self.ex.release(job.handle)
                    self.used -= job.footprint
                    continue
                if job.phase == "grad":  # epoch done: resample
                    job.epoch += 1
                    job.target += job.req.nstep_update
                    job.phase = "sampling"
            keep.append(job)
        self.active = keep
        # jobs whose sampling reached its target: next epoch or the final energy
        for job in self.active:
            if job.phase == "sampling" and job.inflight is None and job.steps_done >= job.target:
                if job.req.kind == "run" and job.epoch < job.req.nepoch:
                    job.phase = "grad"
                    job.inflight = self.ex.launch_epoch(job.handle, job.epoch, self._stream())
                else:
                    job.phase = "energy"
                    job.inflight = self.ex.launch_energy(job.handle, self._stream())
        return out

    def _admit(self):
        while self.queue and len(self.active) < self.max_active:
            req, fp = self.queue[0]
            if self.used + fp > self.budget:
                break
            self.queue.popleft()
            handle, key = self.ex.admit(req)
            self.used += fp
            self._order += 1
            self.active.append(_Job(req, key, fp, self.clock(), handle=handle, order=self._order,
                                    target=req.nstep))

    def _launch(self):
        ready = {}
        for job in self.active:
            if job.phase == "sampling" and job.inflight is None and job.steps_done < job.target:
                ready.setdefault(job.key, []).append(job)
        for key, jobs in ready.items():
            jobs.sort(key=lambda j: j.order)
            for i in range(0, len(jobs), MAX_BATCH):
                chunk = jobs[i:i + MAX_BATCH]
                steps = [min(self.slice_steps, j.target - j.steps_done) for j in chunk]
                token = self.ex.launch_slice([j.handle for j in chunk],
                                             [j.steps_done for j in chunk], steps, self._stream())
                self.launches += 1
                self.launched_jobs += len(chunk)
                for j, n in zip(chunk, steps):
                    j.steps_done += n
                    j.inflight = token


def hydrogen_chain(n, spacing):
    """Linear H_n along z with the given spacing (angstrom), ``Molecule`` syntax."""
    return "; ".join("H 0 0 %.10f" % (i * spacing) for i in range(n))


def seeded_positions(mol, nw, seed):
    """Electrons on their atoms (in ``atomic_nelec`` order) with N(0, 1 bohr^2)
    offsets per coordinate, seeded."""
    rng = np.random.default_rng(seed)
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)[: mol.nelec]
    return (centers[None] + rng.normal(size=(nw, mol.nelec, 3))).reshape(nw, -1)


class GPUExecutor:
    """Device work of the scheduler: wave functions, resident walker state,
    batched Metropolis slices, local energies and statistics."""

    def __init__(self, device=None, nstreams=4):
        import torch

        from . import _lib
        from .wavefunction import runtime as rt
        self.torch = torch
        self.lib = _lib.lib()
        self._lib = _lib
        self.rt = rt
        self.device = device or rt.cuda_device()
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(nstreams)]
        self._mols = {}
        self._sizes = {}
        self._auto = {}
        self._probe_stream = torch.cuda.Stream(device=self.device)

    def _molecule(self, req):
        from .scf import Molecule
        k = (req.atoms, req.unit, req.basis, req.calculator)
        if k not in self._mols:
            self._mols[k] = Molecule(req.atoms, unit=req.unit, basis=req.basis,
                                     calculator=req.calculator)
            if len(self._mols) > 4096:
                self._mols.clear()
        return self._mols[k]

    def precision_of(self, req, mol):
        """(method, probe error) of a request. "auto" takes the mixed method when
        its psi agrees with the FP64 method within AUTO_PSI_TOL relative (median
        over 256 seeded positions of the molecule, probed once per molecule),
        else FP64: the mixed method's FP32 MO values cost about kappa * 6e-8
        relative in each determinant, kappa the Slater matrix's condition
        number, which grows about tenfold per H2 unit of a linear chain."""
        if req.precision != "auto":
            return req.precision, None
        k = (req.atoms, req.unit, req.basis, req.calculator, req.configs)
        if k not in self._auto:
            from .wavefunction import SlaterJastrow
            torch = self.torch
            torch.set_default_dtype(torch.float64)
            self._probe_stream.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(self._probe_stream), torch.no_grad():
                x = torch.as_tensor(seeded_positions(mol, 256, seed=12345), device=self.device)
                p64 = SlaterJastrow(mol, configs=req.configs, cuda=True,
                                    precision="fp64")(x).reshape(-1)
                pm = SlaterJastrow(mol, configs=req.configs, cuda=True,
                                   precision="mixed")(x).reshape(-1)
                err = float(((pm - p64) / p64).abs().median())
            self._auto[k] = ("mixed" if err <= AUTO_PSI_TOL else "fp64", err)
            if len(self._auto) > 4096:
                self._auto.clear()
        return self._auto[k]

    def _wf(self, req, mol):
        from .wavefunction import SlaterJastrow
        self.torch.set_default_dtype(self.torch.float64)
        return SlaterJastrow(mol, configs=req.configs, cuda=True,
                             precision=self.precision_of(req, mol)[0])

    def _shape_key(self, req, mol):
        return (mol.nelec, mol.nup, mol.basis.nao, len(mol.atoms), req.basis, req.configs,
                self.precision_of(req, mol)[0])

    @staticmethod
    def _launch_key(wf):
        """Jobs grouped into one qmc_metropolis_run_batch launch: the same
        precision and MO column class of the determinants (what the kernel
        requires; any molecule otherwise), and electron counts within one band
        of six. A launch runs with the largest job's block size and shared
        memory, so the band keeps the jobs' per-step costs and occupancies
        alike (a small molecule batched with a large one would run at the
        large one's occupancy)."""
        n = wf.highest_occ_mo
        return (wf.precision, 0 if n <= 8 else (1 if n <= 16 else 2),
                (wf.mol.nelec - 1) // 6)

    def footprint(self, req):
        mol = self._molecule(req)
        k = self._shape_key(req, mol)
        if k not in self._sizes:
            wf = self._wf(req, mol)
            call = wf._desc(self.device)
            self._sizes[k] = (call, wf)
        call, _ = self._sizes[k]
        nw = req.nwalkers
        fp = (nw * 3 * mol.nelec * 8                      # positions
              + self.lib.qmc_metropolis_scratch_bytes(call.ref, nw)
              + self.lib.qmc_scratch_bytes(call.ref, nw, 1)  # local energy
              + nw * 8 + self.lib.qmc_reduce_scratch_bytes(nw) + 64)
        if req.kind == "run":  # psi adjoint, psi / weights, parameters with Adam state
            nparam = sum(p.numel() for p in self._sizes[k][1].parameters())
            fp += (self.lib.qmc_adjoint_scratch_bytes(call.ref, nw) + 4 * nw * 8
                   + 4 * nparam * 8 + req.nepoch * 8)
        return int(fp)

    def admit(self, req):
        torch = self.torch
        mol = self._molecule(req)
        wf = self._wf(req, mol)
        call = wf._desc(self.device)
        nw = req.nwalkers
        x = torch.as_tensor(seeded_positions(mol, nw, req.seed), device=self.device)
        h = {
            "req": req, "wf": wf, "call": call, "x": x,
            "met_scr": self.rt.scratch(self.lib.qmc_metropolis_scratch_bytes(call.ref, nw),
                                       self.device),
            "el_scr": self.rt.scratch(self.lib.qmc_scratch_bytes(call.ref, nw, 1), self.device),
            "eloc": torch.empty(nw, dtype=torch.float64, device=self.device),
            "red_scr": self.rt.scratch(self.lib.qmc_reduce_scratch_bytes(nw), self.device),
            "stats": torch.empty(3, dtype=torch.float64, device=self.device),
        }
        if req.kind == "run":
            h["opt"] = torch.optim.Adam(wf.parameters(), lr=req.lr)
            h["energies"] = torch.zeros(max(req.nepoch, 1), dtype=torch.float64,
                                        device=self.device)
        # positions are written on the default stream; the pool streams wait for them
        h["ready"] = torch.cuda.Event()
        h["ready"].record(torch.cuda.current_stream(self.device))
        return h, self._launch_key(wf)

    def _args(self, h, offset, nstep):
        a = self._lib.MetropolisArgs()
        req = h["req"]
        a.pos = self.rt.ptr(h["x"])
        a.nwalkers = req.nwalkers
        a.nstep = nstep
        a.ntherm = nstep
        a.ndecor = 1
        a.move_type = 0
        a.proba = 0
        a.step_size = req.step_size
        a.seed = req.seed
        a.step_offset = offset
        return a

    def launch_slice(self, handles, offsets, steps, sid):
        torch = self.torch
        n = len(handles)
        descs = (self._lib.WfDesc * n)(*[h["call"].desc for h in handles])
        args = (self._lib.MetropolisArgs * n)(*[self._args(h, o, s)
                                                for h, o, s in zip(handles, offsets, steps)])
        scr = (ctypes.c_void_p * n)(*[h["met_scr"].data_ptr() for h in handles])
        nb = (ctypes.c_int64 * n)(*[h["met_scr"].numel() for h in handles])
        stream = self.streams[sid]
        for h in handles:
            stream.wait_event(h["ready"])
        self._lib.check(self.lib.qmc_metropolis_run_batch(descs, args, scr, nb, n,
                                                          ctypes.c_void_p(stream.cuda_stream)),
                        "qmc_metropolis_run_batch")
        ev = torch.cuda.Event()
        ev.record(stream)
        for h in handles:
            h["ready"] = ev
        return ev

    def launch_energy(self, h, sid):
        torch = self.torch
        stream = self.streams[sid]
        stream.wait_event(h["ready"])
        nw = h["req"].nwalkers
        cs = ctypes.c_void_p(stream.cuda_stream)
        self._lib.check(self.lib.qmc_wf_local_energy(
            h["call"].ref, self.rt.ptr(h["x"]), nw, self.rt.ptr(h["eloc"]), None, None,
            self.rt.ptr(h["el_scr"]), h["el_scr"].numel(), cs), "qmc_wf_local_energy")
        self._lib.check(self.lib.qmc_reduce_stats(
            self.rt.ptr(h["eloc"]), nw, self.rt.ptr(h["stats"]), self.rt.ptr(h["red_scr"]),
            h["red_scr"].numel(), cs), "qmc_reduce_stats")
        h["host_stats"] = torch.empty(3, dtype=torch.float64, pin_memory=True)
        with torch.cuda.stream(stream):
            h["host_stats"].copy_(h["stats"], non_blocking=True)
            if h["req"].kind == "run":
                h["host_energies"] = torch.empty(h["energies"].numel(), dtype=torch.float64,
                                                 pin_memory=True)
                h["host_energies"].copy_(h["energies"], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(stream)
        h["ready"] = ev
        return ev

    def launch_epoch(self, h, epoch, sid):
        """One optimisation epoch (solver.py:266-350 with the manual gradient
        of solver.py:372-431): gradient of the energy on the current walkers,
        Adam step; all on the job's stream, no host synchronisation."""
        torch = self.torch
        stream = self.streams[sid]
        stream.wait_event(h["ready"])
        wf, x, opt = h["wf"], h["x"], h["opt"]
        with torch.cuda.stream(stream):
            opt.zero_grad()
            with torch.no_grad():
                eloc = wf.local_energy(x).reshape(-1)
            psi = wf(x).reshape(-1)
            emean = eloc.mean()
            weight = (eloc - emean) / psi.detach() * (2.0 / psi.numel())
            psi.backward(weight)
            opt.step()
            h["energies"][epoch].copy_(emean)
        ev = torch.cuda.Event()
        ev.record(stream)
        h["ready"] = ev
        return ev

    def ready(self, token):
        return token.query()

    def stats(self, h):
        e, v, err = (float(v) for v in h["host_stats"].tolist())
        energies = None
        if h["req"].kind == "run":
            energies = [float(v) for v in h["host_energies"].tolist()][: h["req"].nepoch]
        return e, v, err, energies, self.precision_of(h["req"], h["wf"].mol)

    def release(self, h):
        h.clear()


class VMCServer(Scheduler):
    """The scheduler with the GPU executor: ``submit(Request)``, then
    ``poll()`` / ``run()``; ``results`` maps request ids to ``Result``."""

    def __init__(self, hbm_budget=16 << 30, max_active=256, slice_steps=256, nstreams=4,
                 device=None):
        super().__init__(GPUExecutor(device=device, nstreams=nstreams), hbm_budget,
                         max_active=max_active, slice_steps=slice_steps, nstreams=nstreams)


def single_point(req, device=None):
    """One request alone (no other job on the device)."""
    srv = VMCServer(device=device, nstreams=1)
    srv.submit(req)
    return srv.run()[0]


def poisson_stream(nreq, rate, seed=0, nmin=2, nmax=32, wmin=1024, wmax=16384, smin=100,
                   smax=1000, precision="auto"):
    """Seeded request stream: linear H_n chains (n even in [nmin, nmax],
    spacing uniform in 0.7-1.2 angstrom, sto-3g), walkers log-uniform in
    [wmin, wmax], steps uniform in [smin, smax], Poisson arrival times of the
    given rate (requests/s). Returns [(arrival_s, Request)]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=nreq))
    out = []
    for i in range(nreq):
        n = int(rng.integers(nmin // 2, nmax // 2 + 1)) * 2
        spacing = float(rng.uniform(0.7, 1.2))
        nw = int(round(math.exp(rng.uniform(math.log(wmin), math.log(wmax)))))
        nstep = int(rng.integers(smin, smax + 1))
        out.append((float(t[i]), Request(atoms=hydrogen_chain(n, spacing), nwalkers=nw,
                                         nstep=nstep, seed=1000 + i, precision=precision)))
    return out


def replay_stream(server, stream, clock=time.perf_counter, sleep=2e-4):
    """Submit the requests of ``stream`` at their arrival times (seconds from
    now) while polling ``server``; returns (results, makespan_s)."""
    t0 = clock()
    pending = list(stream)
    out = []
    while pending or not server.idle():
        now = clock() - t0
        while pending and pending[0][0] <= now:
            server.submit(pending.pop(0)[1])
        got = server.poll()
        out += got
        if not got:
            time.sleep(sleep)
    return out, clock() - t0


def latency_percentiles(results, q=(50, 99)):
    lat = np.asarray([r.latency for r in results])
    return {"p%d" % p: float(np.percentile(lat, p)) for p in q}
