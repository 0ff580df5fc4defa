"""Metropolis on an arbitrary density whose tensors live on the GPU: the host
loop of the reference's algorithm (metropolis.py:85-298) runs on the walkers'
CUDA device. The density is a product of normal laws, so the samples must
have its means and variances: per coordinate within 4 sigma of the
statistical error (errors from per-walker means; walkers are independent
chains)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("move", [{"type": "all-elec", "proba": "normal"},
                                  {"type": "one-elec", "proba": "uniform"}])
def test_metropolis_samples_a_cuda_density(move):
    from qmctorch_gb300.sampler import Metropolis
    torch.set_default_dtype(torch.float64)
    rng = np.random.default_rng(3)
    a = torch.as_tensor(rng.uniform(0.4, 1.6, size=6), device="cuda")
    c = torch.as_tensor(rng.uniform(-0.5, 0.5, size=6), device="cuda")

    def pdf(x):
        return torch.exp(-(a * (x - c) ** 2).sum(-1))

    nw, nstep, ntherm, ndecor = 2048, 600, 200, 10
    s = Metropolis(nwalkers=nw, nstep=nstep, step_size=0.8, ntherm=ntherm, ndecor=ndecor,
                   nelec=2, ndim=3, init={"method": "uniform", "min": -1, "max": 1},
                   move=dict(move), cuda=True)
    torch.manual_seed(0)
    x0 = torch.zeros(nw, 6, device="cuda")
    out = s(pdf, pos=x0, with_tqdm=False).detach()
    assert out.device.type == "cpu"  # the reference keeps its snapshots on the host
    nsnap = len(range(ntherm, nstep, ndecor))
    smp = out.reshape(nsnap, nw, 6).numpy()
    wm = smp.mean(0)  # per-walker means
    mean, err = wm.mean(0), wm.std(0, ddof=1) / np.sqrt(nw)
    np.testing.assert_array_less(np.abs(mean - c.cpu().numpy()), 4 * err + 1e-3)
    var = smp.reshape(-1, 6).var(0)
    np.testing.assert_allclose(var, 0.5 / a.cpu().numpy(), rtol=0.06)
    assert 0.05 < s.last_acceptance < 0.95
