"""Stub modules that let the reference QMCTorch package import in a container
that lacks its optional third-party dependencies (twiggy, h5py, matplotlib,
mendeleev, pints, scm.plams, pyscf).

Only the golden-fixture generator in this folder uses this file. The stubs
carry no arithmetic: every number in the fixtures comes from the reference's
own PyTorch code path (wavefunction, sampler, solver)."""
import sys
import types


class _Log:
    def __getattr__(self, name):
        return self

    def __call__(self, *a, **k):
        return self


def _module(name, **attrs):
    mod = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(mod, k, v)
    sys.modules[name] = mod
    return mod


def install(reference_root):
    """Register the stub modules and put the reference on sys.path."""
    log = _Log()
    twiggy = _module("twiggy", quick_setup=lambda **k: None,
                     log=types.SimpleNamespace(name=lambda n: log),
                     levels=types.SimpleNamespace(INFO=20, DEBUG=10))
    del twiggy
    _module("h5py", File=None, Group=object, Dataset=object)
    mpl = _module("matplotlib")
    plt = _module("matplotlib.pyplot")
    cm = _module("matplotlib.cm")
    mpl.pyplot, mpl.cm = plt, cm
    _module("mendeleev", element=None)
    _module("pints", LogPDF=object, MetropolisRandomWalkMCMC=object)
    scm = _module("scm")
    plams = _module("scm.plams", Molecule=object, Settings=object, Atom=object)
    scm.plams = plams
    pyscf = _module("pyscf")
    for sub in ("gto", "scf", "dft"):
        m = _module("pyscf." + sub, M=object, Mole=object, RHF=object, RKS=object)
        setattr(pyscf, sub, m)
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)

    import qmctorch.solver.solver_base as sb
    import qmctorch.solver.solver as sv
    for mod in (sb, sv):
        mod.dump_to_hdf5 = lambda *a, **k: None
        mod.add_group_attr = lambda *a, **k: None
    import qmctorch.utils as qu
    qu.dump_to_hdf5 = lambda *a, **k: None
