"""CPU tests of Solver host logic that needs no kernel: the sampling
trajectory bookkeeping (solver_base.py:435-471) and the optimiser step
dispatch (solver_base.py:486-496), with a stand-in wave function."""
from types import SimpleNamespace

import numpy as np
import torch

from qmctorch_gb300.solver.solver import SolverBase


class _FakeWF(torch.nn.Module):
    def __init__(self):
        super().__init__()
        self.cuda = False
        self.mol = SimpleNamespace(name="fake")
        self.w = torch.nn.Parameter(torch.ones(2))
        self.calls = []

    def pdf(self, x):
        return torch.exp(-(x * x).sum(-1))

    def local_energy(self, x):
        self.calls.append(tuple(x.shape))
        return (x * x).sum(-1, keepdim=True) + 0.5


class _FakeSampler:
    def __init__(self, nwalkers):
        self.walkers = SimpleNamespace(nwalkers=nwalkers, cuda=False)
        self.cuda = False


def test_sampling_traj_evaluates_all_snapshots_in_one_call():
    wf, nw = _FakeWF(), 5
    solver = SolverBase(wf=wf, sampler=_FakeSampler(nw), optimizer=None)
    pos = torch.as_tensor(np.random.default_rng(0).normal(size=(3 * nw, 6)))
    obs = solver.sampling_traj(pos=pos, with_tqdm=False)
    assert wf.calls == [(3 * nw, 6)]
    assert obs.local_energy.shape == (3, nw)
    ref = ((pos * pos).sum(-1) + 0.5).reshape(3, nw).numpy()
    np.testing.assert_allclose(obs.local_energy, ref, rtol=0, atol=0)
    assert obs.pos is pos


class _Opt:
    def __init__(self, lpos_needed):
        self.lpos_needed = lpos_needed
        self.args = None

    def step(self, *args):
        self.args = args


def test_optimization_step_passes_positions_only_when_needed():
    wf = _FakeWF()
    for needed, expect in ((False, 0), (True, 1)):
        opt = _Opt(needed)
        solver = SolverBase(wf=wf, sampler=_FakeSampler(2), optimizer=opt)
        lpos = torch.zeros(2, 6)
        solver.optimization_step(lpos)
        assert len(opt.args) == expect


def test_observable_store_keeps_the_hdf5_tree(tmp_path):
    """dump_observables / add_group_attr / load_observables: the tree of the
    reference's HDF5 dump (hdf5_utils.py:130-160) in an .npz archive, with the
    "_<n>" suffix for a root name already present."""
    from types import SimpleNamespace

    import numpy as np
    import torch

    from qmctorch_gb300.utils import add_group_attr, dump_observables, load_observables
    f = str(tmp_path / "obs.npz")
    obs = SimpleNamespace(energy=[1.0, 2.0, 3.0], local_energy=torch.arange(4.0),
                          models=SimpleNamespace(last={"w": torch.ones(2)}))
    assert dump_observables(obs, f, "wf_opt") == "wf_opt"
    add_group_attr(f, "wf_opt", {"type": "opt"})
    assert dump_observables(obs, f, "wf_opt") == "wf_opt_2"
    back = load_observables(f, "wf_opt")
    np.testing.assert_array_equal(back.energy, [1.0, 2.0, 3.0])
    np.testing.assert_array_equal(back.local_energy, [0, 1, 2, 3])
    np.testing.assert_array_equal(back.models.last.w, [1.0, 1.0])
    assert str(back.attrs["type"]) == "opt"
