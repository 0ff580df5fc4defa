"""VMC solver (drop-in for ``qmctorch.solver.Solver`` / ``SolverBase``,
``qmctorch/solver/solver.py:16-537``, ``solver_base.py:15-546``).

``single_point`` samples with the persistent Metropolis kernel and evaluates
the local energies of all kept samples with the fused local-energy kernel;
mean, variance and error are FP64 reductions of those values. HDF5 output of
the reference is replaced by keeping the observables in memory (h5py is not
part of this package's dependencies).
"""
from __future__ import annotations

import logging
import os
import time
from types import SimpleNamespace

import numpy as np
import torch

from ..utils import DataLoader
from ..wavefunction import runtime as rt
from .loss import Loss

log = logging.getLogger("qmctorch_gb300")


class SolverBase:
    def __init__(self, wf=None, sampler=None, optimizer=None, scheduler=None, output=None,
                 rank=0):
        self.wf = wf
        self.sampler = sampler
        self.opt = optimizer
        self.scheduler = scheduler
        self.cuda = False
        self.device = torch.device("cpu")
        self.dataloader = None
        self.loss = None
        self.obs_dict = None
        if self.opt is not None and "lpos_needed" not in self.opt.__dict__:
            self.opt.lpos_needed = False
        self.save_model = "model.pth"
        if self.wf.cuda:
            self.device = torch.device("cuda")
            self.sampler.cuda = True
            self.sampler.walkers.cuda = True
        self.hdf5file = output
        if output is None:
            self.hdf5file = str(getattr(self.wf.mol, "name", "qmc")) + "_QMCTorch.hdf5"
        # observables go to an .npz archive with the HDF5 file's tree
        # (utils/observable_store.py) when the caller names the output file
        self.dump_file = None
        if output is not None:
            self.dump_file = os.path.splitext(str(output))[0] + ".npz"

    def _dump(self, obs, group, kind):
        """solver_base.py:384-385 / solver.py:262-264: the observables of a
        calculation under ``group`` with its type attribute."""
        if self.dump_file is None:
            return group
        from ..utils import add_group_attr, dump_observables
        group = dump_observables(obs, self.dump_file, root_name=group)
        add_group_attr(self.dump_file, group, {"type": kind})
        return group

    def configure_resampling(self, mode="update", resample_every=1, nstep_update=25,
                             ntherm_update=-1, increment={"every": None, "factor": None}):
        """solver_base.py:74-110."""
        valid = ["never", "full", "update"]
        if mode not in valid:
            raise ValueError(mode, "not a valid update method : ", valid)
        self.resampling_options = SimpleNamespace(mode=mode, resample_every=resample_every,
                                                  ntherm_update=ntherm_update,
                                                  nstep_update=nstep_update, increment=increment)

    def track_observable(self, obs_name):
        """solver_base.py:112-173."""
        if not isinstance(obs_name, list):
            obs_name = [obs_name]
        if "local_energy" not in obs_name:
            obs_name += ["local_energy"]
        self.observable = SimpleNamespace()
        for k in obs_name:
            setattr(self.observable, k, [])
            if k in self.wf.state_dict():
                setattr(self.observable, k + ".grad", [])
        if "energy" not in obs_name:
            self.observable.energy = []
        self.observable.models = SimpleNamespace()

    def store_observable(self, pos, local_energy=None, ibatch=None, **kwargs):
        """solver_base.py:175-248."""
        for obs in list(self.observable.__dict__.keys()):
            if obs == "energy":
                if local_energy is None:
                    local_energy = self.wf.local_energy(pos)
                data = local_energy.detach().cpu().numpy()
                if ibatch is None or ibatch == 0:
                    self.observable.energy.append(np.mean(data).item())
                else:
                    self.observable.energy[-1] *= ibatch / (ibatch + 1)
                    self.observable.energy[-1] += np.mean(data).item() / (ibatch + 1)
            elif obs == "local_energy" and local_energy is not None:
                data = local_energy.detach().cpu().numpy()
                if ibatch is None or ibatch == 0:
                    self.observable.local_energy.append(data)
                else:
                    self.observable.local_energy[-1] = np.append(
                        self.observable.local_energy[-1], data)
            elif obs in self.wf.state_dict():
                p = dict(self.wf.named_parameters()).get(obs)
                val = self.wf.state_dict()[obs]
                getattr(self.observable, obs).append(val.detach().cpu().numpy().copy())
                if obs + ".grad" in self.observable.__dict__:
                    g = p.grad if p is not None else None
                    getattr(self.observable, obs + ".grad").append(
                        (g if g is not None else torch.zeros_like(val)).detach().cpu().numpy())

    def resample(self, n, pos):
        """solver_base.py:273-314."""
        if self.resampling_options.mode != "never":
            if n % self.resampling_options.resample_every == 0:
                if self.resampling_options.mode == "update":
                    pos = pos.clone().detach()[: self.sampler.walkers.nwalkers].to(self.device)
                else:
                    pos = None
                inc = self.resampling_options.increment
                if inc["every"] is not None and n % inc["every"] == 0:
                    self.sampler.nstep += inc["factor"] * self.sampler.ndecor
                pos = self.sampler(self.wf.pdf, pos=pos, with_tqdm=False)
                self.dataloader.dataset = pos
            if self.loss.use_weight:
                self.loss.weight["psi0"] = None
        return pos

    def single_point(self, with_tqdm=True, batchsize=None, hdf5_group="single_point"):
        """Sample, then E_L on every kept sample (solver_base.py:316-387)."""
        log.info("  Single Point Calculation : %d walkers | %d steps",
                 self.sampler.walkers.nwalkers, self.sampler.nstep)
        with torch.no_grad():
            pos = self.sampler(self.wf.pdf, with_tqdm=with_tqdm)
            if self.wf.cuda and pos.device.type == "cpu":
                pos = pos.to(self.device)
            if batchsize is None:
                eloc = self.wf.local_energy(pos)
            else:
                chunks = [self.wf.local_energy(pos[i:i + batchsize])
                          for i in range(0, len(pos), batchsize)]
                eloc = torch.cat(chunks)
            # mean, variance and sampling error: compensated device reduction
            e, s, err = rt.walker_stats(eloc)
        log.info("  Energy   : %f +/- %f", e.item(), err.item())
        log.info("  Variance : %f", s.item())
        log.info("  Size     : %d", len(eloc))
        obs = SimpleNamespace(pos=pos, local_energy=eloc, energy=e, variance=s, error=err)
        self._dump(obs, hdf5_group, "single_point")
        return obs

    def sampling_traj(self, pos=None, with_tqdm=True, hdf5_group="sampling_trajectory"):
        """Local energies along a sampling trajectory (solver_base.py:435-471):
        ``local_energy`` of shape (nsnapshots, nwalkers) as a numpy array and
        the positions. The snapshots are evaluated in one fused local-energy
        call instead of one call per snapshot."""
        log.info("  Sampling trajectory")
        with torch.no_grad():
            if pos is None:
                pos = self.sampler(self.wf.pdf, with_tqdm=with_tqdm)
            nw = self.sampler.walkers.nwalkers
            flat = pos.detach().reshape(-1, pos.shape[-1])
            if self.wf.cuda and flat.device.type == "cpu":
                flat = flat.to(self.device)
            el = self.wf.local_energy(flat).reshape(-1, nw).cpu().numpy()
        obs = SimpleNamespace(local_energy=el, pos=pos)
        self._dump(obs, hdf5_group, "sampling_traj")
        return obs

    def print_parameters(self, grad=False):
        """Print the trainable parameters, or their gradients (solver_base.py:473-484)."""
        for p in self.wf.parameters():
            if p.requires_grad:
                print(p.grad if grad else p)

    def optimization_step(self, lpos):
        """One optimiser step; optimisers that need the positions get them
        (solver_base.py:486-496)."""
        if getattr(self.opt, "lpos_needed", False):
            self.opt.step(lpos)
        else:
            self.opt.step()

    def save_checkpoint(self, epoch, loss):
        filename = "checkpoint_epoch%d.pth" % epoch
        torch.save({"epoch": epoch, "model_state_dict": self.wf.state_dict(),
                    "optimzier_state_dict": self.opt.state_dict(), "loss": loss}, filename)

    def load_checkpoint(self, filename):
        data = torch.load(filename)
        self.wf.load_state_dict(data["model_state_dict"])
        self.opt.load_state_dict(data["optimzier_state_dict"])
        return data["epoch"], data["loss"]


class Solver(SolverBase):
    def __init__(self, wf=None, sampler=None, optimizer=None, scheduler=None, output=None,
                 rank=0):
        SolverBase.__init__(self, wf, sampler, optimizer, scheduler, output, rank)
        self.set_params_requires_grad()
        self.configure(track=["local_energy"], freeze=None, loss="energy", grad="manual",
                       ortho_mo=False, clip_loss=False,
                       resampling={"mode": "update", "resample_every": 1, "nstep_update": 25})

    def configure(self, track=None, freeze=None, loss=None, grad=None, ortho_mo=None,
                  clip_loss=False, clip_threshold=5, resampling=None):
        """solver.py:50-111."""
        self.set_params_requires_grad()
        self.freeze_params_list = freeze
        self.freeze_parameters(freeze)
        if track is not None:
            self.track_observable(track)
        if grad is not None:
            self.grad_method = grad
            self.evaluate_gradient = {"auto": self.evaluate_grad_auto,
                                      "manual": self.evaluate_grad_manual}[grad]
        if resampling is not None:
            self.configure_resampling(**resampling)
        if loss is not None:
            self.loss = Loss(self.wf, method=loss, clip=clip_loss, clip_threshold=clip_threshold)
            self.loss.use_weight = self.resampling_options.resample_every > 1
        self.ortho_mo = ortho_mo

    def set_params_requires_grad(self, wf_params=True, geo_params=False):
        """solver.py:113-134."""
        self.wf.ao.bas_exp.requires_grad = wf_params
        for param in self.wf.mo.parameters():
            param.requires_grad = wf_params
        self.wf.fc.weight.requires_grad = wf_params
        if getattr(self.wf, "jastrow", None) is not None:
            for param in self.wf.jastrow.parameters():
                param.requires_grad = wf_params
        self.wf.ao.atom_coords.requires_grad = geo_params

    def freeze_parameters(self, freeze):
        """solver.py:136-167."""
        if freeze is None:
            return
        if not isinstance(freeze, list):
            freeze = [freeze]
        for name in freeze:
            n = name.lower()
            if n == "ci":
                self.wf.fc.weight.requires_grad = False
            elif n == "mo":
                for param in self.wf.mo.parameters():
                    param.requires_grad = False
            elif n == "ao":
                self.wf.ao.bas_exp.requires_grad = False
            elif n == "jastrow":
                for param in self.wf.jastrow.parameters():
                    param.requires_grad = False
            else:
                raise ValueError("Valid arguments for freeze are :",
                                 ["ci", "mo", "ao", "jastrow", "backflow"])

    def save_sampling_parameters(self):
        self.sampler._nstep_save = self.sampler.nstep
        self.sampler._ntherm_save = self.sampler.ntherm
        if self.resampling_options.mode == "update":
            self.sampler.ntherm = self.resampling_options.ntherm_update
            self.sampler.nstep = self.resampling_options.nstep_update

    def restore_sampling_parameters(self):
        self.sampler.nstep = self.sampler._nstep_save
        self.sampler.ntherm = self.sampler._ntherm_save

    def run(self, nepoch, batchsize=None, hdf5_group="wf_opt", chkpt_every=None, tqdm=False):
        """Wave-function optimisation (solver.py:186-219)."""
        self.prepare_optimization(batchsize, chkpt_every, tqdm)
        self.run_epochs(nepoch)
        self.restore_sampling_parameters()
        self.observable.models.last = dict(self.wf.state_dict())
        self._dump(self.observable, hdf5_group, "opt")
        return self.observable

    def prepare_optimization(self, batchsize, chkpt_every, tqdm=False):
        """solver.py:221-252."""
        tstart = time.time()
        pos = self.sampler(self.wf.pdf, with_tqdm=tqdm)
        if batchsize is None:
            batchsize = len(pos)
        self.save_sampling_parameters()
        self.dataloader = DataLoader(pos.detach(), batch_size=batchsize, pin_memory=False)
        for ibatch, data in enumerate(self.dataloader):
            self.store_observable(data, ibatch=ibatch)
        self.chkpt_every = chkpt_every
        log.info("  done in %1.2f sec.", time.time() - tstart)

    def run_epochs(self, nepoch, with_tqdm=False, verbose=True):
        """solver.py:266-350."""
        cumulative_loss = 0
        min_loss = 0
        for n in range(nepoch):
            tstart = time.time()
            cumulative_loss = 0
            self.opt.zero_grad()
            self.wf.zero_grad()
            for ibatch, data in enumerate(self.dataloader):
                lpos = data.to(self.device)
                loss, eloc = self.evaluate_gradient(lpos)
                cumulative_loss += loss.item()
                if torch.isnan(eloc).any():
                    log.info("Error : Nan detected in local energy")
                    return cumulative_loss
                self.store_observable(lpos, local_energy=eloc, ibatch=ibatch)
            self.optimization_step(lpos)
            if n == 0 or cumulative_loss < min_loss:
                min_loss = cumulative_loss
                self.observable.models.best = dict(self.wf.state_dict())
            if self.chkpt_every is not None and n > 0 and n % self.chkpt_every == 0:
                self.save_checkpoint(n, cumulative_loss)
            self.dataloader.dataset = self.resample(n, self.dataloader.dataset)
            if self.scheduler is not None:
                self.scheduler.step()
            if verbose:
                log.info("  epoch %d done in %1.2f sec. energy %f", n, time.time() - tstart,
                         self.observable.energy[-1] if self.observable.energy else float("nan"))
        return cumulative_loss

    def evaluate_grad_auto(self, lpos):
        """solver.py:352-370: gradient of the loss through the local energy
        (hand-written local-energy adjoint behind wf.local_energy)."""
        loss, eloc = self.loss(lpos)
        loss.backward()
        return loss, eloc

    def evaluate_grad_manual(self, lpos):
        """solver.py:372-431: dE/dk = 2 < (E_L - <E_L>) dpsi/dk / psi >."""
        if self.loss.method not in ["energy", "weighted-energy"]:
            raise ValueError("Manual gradient only for energy minimization")
        with torch.no_grad():
            eloc = self.wf.local_energy(lpos)
        psi = self.wf(lpos)
        norm = 1.0 / len(psi)
        weight = eloc.clone()
        weight -= torch.mean(eloc)
        weight /= psi.clone()
        weight *= 2.0 * norm
        clip_mask = self.loss.get_clipping_mask(eloc)
        psi = psi[clip_mask]
        weight = weight[clip_mask]
        psi.backward(weight)
        return torch.mean(eloc), eloc
