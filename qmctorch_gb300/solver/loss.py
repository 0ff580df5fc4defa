"""Loss of the wave-function optimisation (drop-in for
``qmctorch.solver.loss.Loss``, ``qmctorch/solver/loss.py:7-145``).

Behaviour (the contract the solver relies on):

* ``E`` = local energies of the batch, ``w`` = sampling weights, ``m`` = the
  clip mask; the loss is ``reduce(w * E)`` over the entries where ``m`` holds,
  ``reduce`` = mean (``method="energy"``) or unbiased variance
  (``method="variance"``); any other method raises ``KeyError``.
* clipping off: every entry is kept; on: entries whose distance to the median
  exceeds ``clip_threshold`` standard deviations are dropped.
* weights (only while ``use_weight`` holds and the call does not deactivate
  them): ``psi = wf(pos)`` is stored in ``weight["psi"]``; the first call after
  a resampling (``weight["psi0"] is None``) stores a detached copy as the
  reference ``psi0`` and uses unit weights; later calls use
  ``(psi / psi0)^2`` normalised to sum 1. Without weights the factor is the
  scalar 1.
"""
from __future__ import annotations

import torch
from torch import nn

_REDUCTIONS = {"energy": torch.mean, "variance": torch.var}


def _within_spread(values, nstd):
    """True where |values - median| < nstd * std(values)."""
    centre = torch.median(values)
    spread = torch.std(values)
    return ((values - centre) / spread).abs() < nstd


class Loss(nn.Module):
    def __init__(self, wf, method="energy", clip=False, clip_threshold=5):
        super().__init__()
        self.loss_fn = _REDUCTIONS[method]
        self.wf = wf
        self.method = method
        self.clip = clip
        self.clip_num_std = clip_threshold
        self.use_weight = True
        self.weight = {"psi": None, "psi0": None}

    def forward(self, pos, no_grad=False, deactivate_weight=False):
        """Returns (loss, local energies) of the batch ``pos``."""
        with self.get_grad_mode(no_grad):
            eloc = self.wf.local_energy(pos)
            keep = self.get_clipping_mask(eloc)
            factor = self.get_sampling_weights(pos, deactivate_weight)
            weighted = factor * eloc
            return self.loss_fn(weighted[keep]), eloc

    @staticmethod
    def get_grad_mode(no_grad):
        """Context manager: autograd off when ``no_grad``."""
        if no_grad:
            return torch.no_grad()
        return torch.enable_grad()

    def get_clipping_mask(self, local_energies):
        """Boolean mask of the local energies the loss keeps."""
        if not self.clip:
            return torch.ones_like(local_energies, dtype=torch.bool)
        return _within_spread(local_energies, self.clip_num_std)

    def get_sampling_weights(self, pos, deactivate_weight):
        """Reweighting of samples drawn from an earlier wave function."""
        if not (self.use_weight and not deactivate_weight):
            return torch.tensor(1.0)
        psi = self.wf(pos)
        self.weight["psi"] = psi
        if self.weight["psi0"] is None:  # just resampled: psi is the sampling density
            self.weight["psi0"] = psi.detach().clone()
            return torch.ones_like(psi)
        ratio2 = (psi / self.weight["psi0"]) ** 2
        return ratio2 / ratio2.sum()
