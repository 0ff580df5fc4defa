"""Product of Jastrow factors (drop-in for ``CombineJastrow``,
``qmctorch/wavefunction/jastrows/combine_jastrow.py:7-195``).

J = prod_k J_k. Derivatives by the product rule on the factors' own outputs:
grad J = sum_k grad J_k prod_{m != k} J_m and
lap J = sum_k lap J_k prod_{m != k} J_m
        + 2 sum_{k < l} (grad J_k . grad J_l) prod_{m != k, l} J_m.
As in the reference, ``derivative=[0, 1, 2]`` returns the per-axis gradient
(sum_grad is not applied). Inside a wave function the factors are fused into
the kernels (log J = sum_k log J_k); this module is the standalone call.
"""
from __future__ import annotations

from functools import reduce

from torch import nn


def _prod(vals):
    return reduce(lambda a, b: a * b, vals)


def _others(vals, skip):
    """Product of vals without the entries whose index is in ``skip`` (or 1)."""
    rest = [v for i, v in enumerate(vals) if i not in skip]
    return _prod(rest) if rest else 1.0


class CombineJastrow(nn.Module):
    def __init__(self, jastrow):
        super().__init__()
        self.jastrow_terms = nn.ModuleList(list(jastrow))
        self.requires_autograd = True
        self.nterms = len(self.jastrow_terms)

    def __repr__(self):
        return " + ".join(repr(t) for t in self.jastrow_terms)

    def forward(self, pos, derivative=0, sum_grad=True):
        terms = self.jastrow_terms
        if derivative == 0:
            return self.get_combined_values([t(pos) for t in terms])
        if derivative == 1:
            vals = [t(pos) for t in terms]
            if not sum_grad:
                vals = [v.unsqueeze(-1) for v in vals]
            grads = [t(pos, derivative=1, sum_grad=sum_grad) for t in terms]
            return self.get_derivative_combined_values(vals, grads)
        if derivative == 2:
            vals = [t(pos) for t in terms]
            grads = [t(pos, derivative=1, sum_grad=False) for t in terms]
            laps = [t(pos, derivative=2) for t in terms]
            return self.get_second_derivative_combined_values(vals, grads, laps)
        if derivative == [0, 1, 2]:
            vals = [t(pos) for t in terms]
            grads = [t(pos, derivative=1, sum_grad=False) for t in terms]
            laps = [t(pos, derivative=2) for t in terms]
            lap = self.get_second_derivative_combined_values(vals, grads, laps)
            grad = self.get_derivative_combined_values([v.unsqueeze(-1) for v in vals], grads)
            return self.get_combined_values(vals), grad, lap
        raise ValueError("derivative not understood")

    @staticmethod
    def get_combined_values(jast_vals):
        """prod_k J_k."""
        return _prod(jast_vals)

    @staticmethod
    def get_derivative_combined_values(jast_vals, djast_vals):
        """sum_k grad J_k prod_{m != k} J_m."""
        if len(djast_vals) == 1:
            return djast_vals[0]
        return sum(g * _others(jast_vals, {k}) for k, g in enumerate(djast_vals))

    @staticmethod
    def get_second_derivative_combined_values(jast_vals, djast_vals, d2jast_vals):
        """sum_k lap J_k prod_{m != k} J_m + 2 sum_{k<l} (grad J_k . grad J_l) prod_{others}."""
        if len(d2jast_vals) == 1:
            return d2jast_vals[0]
        out = sum(h * _others(jast_vals, {k}) for k, h in enumerate(d2jast_vals))
        wide = [v.unsqueeze(-1) for v in jast_vals]  # (nb, 1, 1) against (nb, 3, ne)
        n = len(jast_vals)
        for k in range(n - 1):
            for m in range(k + 1, n):
                cross = djast_vals[k] * djast_vals[m] * _others(wide, {k, m})
                out = out + 2.0 * cross.sum(1)
        return out
