"""Loss of the wave-function optimisation (drop-in for
``qmctorch.solver.loss.Loss``, ``qmctorch/solver/loss.py:7-145``)."""
from __future__ import annotations

import torch
from torch import nn


class Loss(nn.Module):
    def __init__(self, wf, method="energy", clip=False, clip_threshold=5):
        super().__init__()
        self.wf = wf
        self.method = method
        self.clip = clip
        self.use_weight = True
        self.clip_num_std = clip_threshold
        self.loss_fn = {"energy": torch.mean, "variance": torch.var}[method]
        self.weight = {"psi": None, "psi0": None}

    def forward(self, pos, no_grad=False, deactivate_weight=False):
        with self.get_grad_mode(no_grad):
            local_energies = self.wf.local_energy(pos)
            mask = self.get_clipping_mask(local_energies)
            weight = self.get_sampling_weights(pos, deactivate_weight)
            loss = self.loss_fn((weight * local_energies)[mask])
        return loss, local_energies

    @staticmethod
    def get_grad_mode(no_grad):
        return torch.no_grad() if no_grad else torch.enable_grad()

    def get_clipping_mask(self, local_energies):
        if self.clip:
            median = torch.median(local_energies)
            std = torch.std(local_energies)
            zscore = torch.abs((local_energies - median) / std)
            return zscore < self.clip_num_std
        return torch.ones_like(local_energies).type(torch.bool)

    def get_sampling_weights(self, pos, deactivate_weight):
        if self.use_weight * (not deactivate_weight):
            self.weight["psi"] = self.wf(pos)
            if self.weight["psi0"] is None:
                self.weight["psi0"] = self.weight["psi"].detach().clone()
                return torch.ones_like(self.weight["psi"])
            w = (self.weight["psi"] / self.weight["psi0"]) ** 2
            return w / w.sum()
        return torch.tensor(1.0)
