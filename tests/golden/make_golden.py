"""Generate the golden fixtures of the VMC hot path by running the reference
QMCTorch package itself (FP64, CPU) on seeded inputs.

Usage (in a container where the reference source tree is available):

    python tests/golden/make_golden.py /path/to/QMCTorch [case ...]

The reference root may also come from the environment variable
``QMCTORCH_REFERENCE`` (then every argument is a case name).

Writes ``tests/golden/<case>.npz``. Each file holds the molecule / basis
namespace (``mol_*`` / ``basis_*`` keys, the layout of
``qmctorch_gb300.scf.Molecule.save``), the seeded walker positions and the
reference outputs: AO values and derivatives, MOs, Jastrow factor and
derivatives, Slater determinants, psi, pdf, their electron-position
gradients (gradients_jacobi), kinetic and local energies, a
Metropolis replay with injected proposals and uniforms, and the parameter
gradients of the manual and automatic VMC energy gradients. ``gmetropolis``
writes ``tests/golden/gmetropolis.npz``: chains of the reference's
GeneralizedMetropolis (drift-diffusion) sampler on an analytic density.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import ref_stubs  # noqa: E402

CASES = {
    # name: (atoms, unit, basis, configs, include_all_mo, nwalkers, random_ci, extras)
    "h2": ("H 0 0 -0.37; H 0 0 0.37", "angs", "sto-3g", "ground_state", True, 12, False,
           ("metropolis", "solver")),
    "lih_cas": ("Li 0 0 0; H 0 0 1.595", "angs", "sto-3g", "cas(2,2)", True, 12, True,
                ("metropolis", "solver")),
    "lih_sd": ("Li 0 0 0; H 0 0 3.14", "bohr", "sto-3g", "single_double(2,2)", False, 11, True,
               ("solver",)),
    "h2o_sd": ("O 0 0 0.1173; H 0 0.7572 -0.4692; H 0 -0.7572 -0.4692", "angs", "cc-pvdz",
               "single_double(4,4)", True, 8, True, ("metropolis", "iter", "solver")),
    "h2o_single": ("O 0 0 0.1173; H 0 0.7572 -0.4692; H 0 -0.7572 -0.4692", "angs", "cc-pvdz",
                   "single(2,2)", True, 6, True, ()),
    "h4": ("H 0 0 0; H 0 0 1.0; H 0 0 2.0; H 0 0 3.0", "angs", "sto-3g", "ground_state",
           False, 8, False, ("metropolis", "iter", "oneelec")),
    "c6h6": ("C 1.39 0 0; C 0.695 1.20377 0; C -0.695 1.20377 0; C -1.39 0 0; "
             "C -0.695 -1.20377 0; C 0.695 -1.20377 0; H 2.48 0 0; H 1.24 2.14774 0; "
             "H -1.24 2.14774 0; H -2.48 0 0; H -1.24 -2.14774 0; H 1.24 -2.14774 0",
             "angs", "cc-pvdz", "ground_state", True, 3, False, ("iter", "oneelec")),
}


# Jastrow factors of the cases that do not use the default e-e Pade factor:
# "ee+en" = CombineJastrow([e-e Pade, e-n Pade]) (combine_jastrow.py:7-195),
# "en" = the e-n Pade factor alone (jastrow_factor_electron_nuclei.py:9-161),
# with the kernels' initial weights (w of each Pade kernel).
JASTROW = {"lih_en": ("ee+en", 1.0, 0.8), "h2o_en": ("ee+en", 1.0, 1.3),
           "h2_en": ("en", None, 0.6), "c6h6_en": ("ee+en", 2.0, 10.0)}
CASES.update({
    "lih_en": ("Li 0 0 0; H 0 0 1.595", "angs", "sto-3g", "cas(2,2)", True, 12, True,
               ("metropolis", "solver")),
    "h2o_en": ("O 0 0 0.1173; H 0 0.7572 -0.4692; H 0 -0.7572 -0.4692", "angs", "cc-pvdz",
               "single_double(4,4)", True, 8, True, ("metropolis", "iter", "solver")),
    "h2_en": ("H 0 0 -0.37; H 0 0 0.37", "angs", "sto-3g", "ground_state", True, 12, False,
              ("metropolis", "solver")),
    "c6h6_en": (CASES["c6h6"][0], "angs", "cc-pvdz", "ground_state", True, 3, False,
                ("iter", "oneelec")),
})


# Slater-type orbital cases: the "slater-sz" basis in the ADF calculator's
# layout (radial_type "sto", cartesian harmonics, kr powers of r).
CASES.update({
    "lih_sto": ("Li 0 0 0; H 0 0 1.595", "angs", "slater-sz", "cas(2,2)", True, 10, True,
                ("metropolis", "solver")),
    "h2o_sto": ("O 0 0 0.1173; H 0 0.7572 -0.4692; H 0 -0.7572 -0.4692", "angs", "slater-sz",
                "single_double(2,2)", True, 8, True, ("metropolis", "solver")),
})
# MO source of each case: the fixtures of Gaussian bases were written with
# the extended-Hueckel orbitals, those of the Slater basis with its synthetic ones
CALCULATOR = {"lih_sto": "slater", "h2o_sto": "slater"}


def make_jastrow(mol, name):
    """The reference Jastrow object of a case (None: the default e-e factor)."""
    if name not in JASTROW:
        return "default"
    from qmctorch.wavefunction.jastrows.elec_elec import JastrowFactor as JEE
    from qmctorch.wavefunction.jastrows.elec_elec import PadeJastrowKernel as PEE
    from qmctorch.wavefunction.jastrows.elec_nuclei import JastrowFactor as JEN
    from qmctorch.wavefunction.jastrows.elec_nuclei import PadeJastrowKernel as PEN
    kind, w_ee, w_en = JASTROW[name]
    en = JEN(mol, PEN, kernel_kwargs={"w": w_en})
    if kind == "en":
        return en
    return [JEE(mol, PEE, kernel_kwargs={"w": w_ee}), en]


def seeded_positions(mol, nw, seed):
    """Electrons assigned to atoms in order of their electron count, offset by
    N(0, 1 bohr^2) per coordinate."""
    rng = np.random.default_rng(seed)
    centers = []
    for iat, ne in enumerate(mol.atomic_nelec):
        centers += [mol.atom_coords[iat]] * ne
    centers = np.asarray(centers[: mol.nelec])
    pos = centers[None] + rng.normal(size=(nw, mol.nelec, 3))
    return pos.reshape(nw, -1)


def main(reference_root, only=()):
    ref_stubs.install(reference_root)
    import torch
    from qmctorch.utils import set_torch_double_precision
    from qmctorch.wavefunction import SlaterJastrow
    from qmctorch.sampler import Metropolis
    from qmctorch.solver import Solver
    import qmctorch.sampler.metropolis as qmet
    from qmctorch_gb300.scf import Molecule

    set_torch_double_precision()
    for name, (atoms, unit, basis, configs, all_mo, nw, random_ci, extras) in CASES.items():
        if only and name not in only:
            continue
        torch.manual_seed(1234)
        mol = Molecule(atoms, unit=unit, basis=basis, calculator=CALCULATOR.get(name, "huckel"))
        tmp = os.path.join(HERE, "_tmp_mol.npz")
        mol.save(tmp)
        data = dict(np.load(tmp))
        os.remove(tmp)
        wf = SlaterJastrow(mol, configs=configs, include_all_mo=all_mo,
                           jastrow=make_jastrow(mol, name))
        if random_ci:
            g = torch.Generator().manual_seed(7)
            wf.fc.weight.data = torch.rand(wf.fc.weight.shape, generator=g)
        pos_np = seeded_positions(mol, nw, seed=11)
        pos = torch.as_tensor(pos_np)
        data.update(case_configs=np.asarray(configs), case_include_all_mo=np.asarray(all_mo),
                    fc_weight=wf.fc.weight.detach().numpy().reshape(-1),
                    pos=pos_np)
        if name in JASTROW:
            data.update(case_jastrow=np.asarray(JASTROW[name][0]))
            for pname, p in wf.named_parameters():
                if pname.startswith("jastrow."):
                    data["param_" + pname] = p.detach().numpy().copy()
        else:
            data.update(jastrow_w=wf.jastrow.jastrow_kernel.weight.detach().numpy())
        with torch.no_grad():
            if not name.startswith("c6h6"):
                ao, dao, d2ao = wf.ao(pos, derivative=[0, 1, 2])
                data.update(ao=ao.numpy(), dao=dao.numpy(), d2ao=d2ao.numpy(),
                            ao_sumgrad=wf.ao(pos, derivative=1).numpy(),
                            mo=wf.mo(ao).numpy())
                jast, djast, d2jast = wf.jastrow(pos, derivative=[0, 1, 2], sum_grad=False)
                data.update(jast=jast.numpy(), djast=djast.numpy(), d2jast=d2jast.numpy(),
                            djast_sum=wf.jastrow(pos, derivative=1).numpy(),
                            dets=wf.pool(wf.mo(ao)).numpy())
            data.update(grad_psi=wf.gradients_jacobi(pos).numpy(),
                        grad_pdf=wf.gradients_jacobi(pos, pdf=True).numpy())
            data.update(psi=wf(pos).numpy(), pdf=wf.pdf(pos).numpy(),
                        kinetic=wf.kinetic_energy(pos).numpy(),
                        eloc=wf.local_energy(pos).numpy(),
                        v_en=wf.nuclear_potential(pos).numpy(),
                        v_ee=wf.electronic_potential(pos).numpy(),
                        v_nn=np.asarray(float(wf.nuclear_repulsion())))

        if "metropolis" in extras:
            rng = np.random.default_rng(21)
            mnw, nstep, step = 8, 12, 0.2
            sig = np.sqrt(step / (2 * np.sqrt(2 * np.log(2))))
            props = rng.normal(size=(nstep, mnw, 3 * mol.nelec)) * sig
            unif = rng.uniform(size=(nstep, mnw))
            pos0 = seeded_positions(mol, mnw, seed=5)
            sampler = Metropolis(nwalkers=mnw, nstep=nstep, step_size=step, ntherm=4,
                                 ndecor=2, nelec=mol.nelec, init=mol.domain("atomic"),
                                 move={"type": "all-elec", "proba": "normal"})
            it_p = iter(torch.as_tensor(props))
            it_u = iter(torch.as_tensor(unif))
            sampler._move = types.MethodType(lambda self, n: next(it_p), sampler)
            orig = qmet.torch.rand_like
            qmet.torch.rand_like = lambda t: next(it_u).reshape(t.shape).type(t.dtype)
            try:
                out = sampler(wf.pdf, pos=torch.tensor(pos0), with_tqdm=False)
            finally:
                qmet.torch.rand_like = orig
            data.update(met_pos0=pos0, met_props=props, met_unif=unif,
                        met_step=np.asarray(step), met_ntherm=np.asarray(4),
                        met_ndecor=np.asarray(2), met_out=out.detach().numpy())

        if "iter" in extras:
            rng = np.random.default_rng(22)
            mnw, nstep, step = 6, 3, 0.3
            sig = np.sqrt(step / (2 * np.sqrt(2 * np.log(2))))
            props = rng.normal(size=(nstep, mol.nelec, mnw, 3)) * sig
            unif = rng.uniform(size=(nstep, mol.nelec, mnw))
            pos0 = seeded_positions(mol, mnw, seed=6)
            sampler = Metropolis(nwalkers=mnw, nstep=nstep, step_size=step, ntherm=-1,
                                 ndecor=1, nelec=mol.nelec, init=mol.domain("atomic"),
                                 move={"type": "all-elec-iter", "proba": "normal"})
            it_p = iter(torch.as_tensor(props.reshape(nstep * mol.nelec, mnw, 3)))
            it_u = iter(torch.as_tensor(unif.reshape(nstep * mol.nelec, mnw)))
            sampler._move = types.MethodType(lambda self, n: next(it_p), sampler)
            orig = qmet.torch.rand_like
            qmet.torch.rand_like = lambda t: next(it_u).reshape(t.shape).type(t.dtype)
            try:
                out = sampler(wf.pdf, pos=torch.tensor(pos0), with_tqdm=False)
            finally:
                qmet.torch.rand_like = orig
            data.update(iter_pos0=pos0, iter_props=props, iter_unif=unif,
                        iter_out=out.detach().numpy())

        if "oneelec" in extras:
            rng = np.random.default_rng(23)
            mnw, nstep, step = 6, 10, 0.3
            sig = np.sqrt(step / (2 * np.sqrt(2 * np.log(2))))
            props = rng.normal(size=(nstep, mnw, 3)) * sig
            unif = rng.uniform(size=(nstep, mnw))
            pos0 = seeded_positions(mol, mnw, seed=7)
            sampler = Metropolis(nwalkers=mnw, nstep=nstep, step_size=step, ntherm=2,
                                 ndecor=3, nelec=mol.nelec, init=mol.domain("atomic"),
                                 move={"type": "one-elec", "proba": "normal"})
            it_p = iter(torch.as_tensor(props))
            it_u = iter(torch.as_tensor(unif))
            sampler._move = types.MethodType(lambda self, n: next(it_p), sampler)
            orig = qmet.torch.rand_like
            qmet.torch.rand_like = lambda t: next(it_u).reshape(t.shape).type(t.dtype)
            # the electron indices are the only draws left on torch's generator
            torch.manual_seed(99)
            try:
                out = sampler(wf.pdf, pos=torch.tensor(pos0), with_tqdm=False)
            finally:
                qmet.torch.rand_like = orig
            torch.manual_seed(99)
            index = np.stack([torch.LongTensor(mnw).random_(0, mol.nelec).numpy()
                              for _ in range(nstep)])
            data.update(one_pos0=pos0, one_props=props, one_unif=unif, one_index=index,
                        one_step=np.asarray(step), one_ntherm=np.asarray(2),
                        one_ndecor=np.asarray(3), one_out=out.detach().numpy())

        if "solver" in extras:
            sampler = Metropolis(nwalkers=nw, nstep=2, step_size=0.2, nelec=mol.nelec,
                                 init=mol.domain("atomic"))
            opt = torch.optim.Adam(wf.parameters(), lr=1e-3)
            solver = Solver(wf=wf, sampler=sampler, optimizer=opt, output="_unused.hdf5")
            names = ["ao.bas_exp", "mo.mo_modifier", "jastrow.jastrow_kernel.weight",
                     "fc.weight"]
            params = dict(wf.named_parameters())
            if name in JASTROW:
                names = [n for n in params if n != "ao.atom_coords"]
            for mode in ("manual", "auto"):
                solver.configure(grad=mode, loss="energy", track=["local_energy"])
                solver.loss.use_weight = False
                opt.zero_grad()
                wf.zero_grad()
                lpos = pos.clone().requires_grad_(mode == "auto")
                loss, eloc = solver.evaluate_gradient(lpos)
                data["grad_%s_loss" % mode] = np.asarray(float(loss))
                for n in names:
                    g = params[n].grad
                    data["grad_%s_%s" % (mode, n)] = (np.zeros(params[n].shape) if g is None
                                                      else g.detach().numpy().copy())
        out_file = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out_file, **data)
        print("wrote", out_file, os.path.getsize(out_file), "bytes")


# Drift-diffusion (generalized Metropolis) chains of the reference sampler on
# an analytic density: rho(x) = exp(-sum_k a_k (x_k - c_k)^2) over the flattened
# walker coordinates, drift by the reference's own autograd (get_drift).
GMET = {"nwalkers": 24, "nelec": 2, "ndim": 3, "nstep": 30, "step_size": 0.3,
        "ntherm": -10, "ndecor": 2, "seed": 2024}


def gmet_density_params():
    rng = np.random.default_rng(5)
    n = GMET["nelec"] * GMET["ndim"]
    return rng.uniform(0.4, 1.6, size=n), rng.uniform(-0.5, 0.5, size=n)


def make_gmetropolis(reference_root):
    ref_stubs.install(reference_root)
    import torch
    from qmctorch.sampler.generalized_metropolis import GeneralizedMetropolis
    from qmctorch.utils import set_torch_double_precision

    set_torch_double_precision()
    a, c = gmet_density_params()
    at, ct = torch.as_tensor(a), torch.as_tensor(c)

    def pdf(x):
        return torch.exp(-(at * (x - ct) ** 2).sum(-1))

    pos0 = np.random.default_rng(6).normal(size=(GMET["nwalkers"], GMET["nelec"] * GMET["ndim"]))
    g = GMET
    sampler = GeneralizedMetropolis(nwalkers=g["nwalkers"], nstep=g["nstep"],
                                    step_size=g["step_size"], ntherm=g["ntherm"],
                                    ndecor=g["ndecor"], nelec=g["nelec"], ndim=g["ndim"],
                                    init={"method": "uniform", "min": -1, "max": 1})
    torch.manual_seed(g["seed"])
    samples = sampler(pdf, pos=torch.as_tensor(pos0), with_tqdm=False)
    # the same sampler on the H2 sto-3g SlaterJastrow of the "h2" case
    from qmctorch.wavefunction import SlaterJastrow
    from qmctorch_gb300.scf import Molecule
    atoms, unit, basis, configs, all_mo = CASES["h2"][:5]
    torch.manual_seed(1234)
    mol = Molecule(atoms, unit=unit, basis=basis, calculator="huckel")
    wf = SlaterJastrow(mol, configs=configs, include_all_mo=all_mo)
    h2pos0 = seeded_positions(mol, 16, seed=21)
    hs = GeneralizedMetropolis(nwalkers=16, nstep=20, step_size=0.2, ntherm=-10, ndecor=2,
                               nelec=mol.nelec, ndim=3,
                               init={"method": "uniform", "min": -1, "max": 1})
    torch.manual_seed(g["seed"] + 1)
    h2samples = hs(wf.pdf, pos=torch.as_tensor(h2pos0), with_tqdm=False)
    out_file = os.path.join(HERE, "gmetropolis.npz")
    np.savez_compressed(out_file, a=a, c=c, pos0=pos0, samples=samples.detach().numpy(),
                        final=sampler.walkers.pos.detach().numpy(),
                        h2_pos0=h2pos0, h2_samples=h2samples.detach().numpy(),
                        h2_final=hs.walkers.pos.detach().numpy(),
                        **{"cfg_" + k: np.asarray(v) for k, v in GMET.items()})
    print("wrote", out_file, os.path.getsize(out_file), "bytes")


# Walker initialisation of the reference (walkers.py:41-150): positions drawn
# with torch's and numpy's global generators seeded before each call.
WALKER_CASES = ("h2o_sd", "lih_cas")
WALKER_METHODS = ("atomic", "center", "uniform", "normal")
WALKER_SEEDS = (31, 32)  # torch.manual_seed, np.random.seed
WALKER_NW = 40


def make_walkers(reference_root):
    ref_stubs.install(reference_root)
    import torch
    from qmctorch.sampler.walkers import Walkers
    from qmctorch.utils import set_torch_double_precision
    from qmctorch_gb300.scf import Molecule

    set_torch_double_precision()
    out = {}
    for name in WALKER_CASES:
        atoms, unit, basis = CASES[name][:3]
        mol = Molecule(atoms, unit=unit, basis=basis, calculator="huckel")
        for method in WALKER_METHODS:
            torch.manual_seed(WALKER_SEEDS[0])
            np.random.seed(WALKER_SEEDS[1])
            w = Walkers(nwalkers=WALKER_NW, nelec=mol.nelec, ndim=3, init=mol.domain(method))
            w.initialize()
            out["%s_%s" % (name, method)] = w.pos.detach().numpy()
    out_file = os.path.join(HERE, "walkers.npz")
    np.savez_compressed(out_file, **out)
    print("wrote", out_file, os.path.getsize(out_file), "bytes")


# Chains of the reference Metropolis sampler on an arbitrary density (the
# analytic one of the drift-diffusion fixture): every move type, both proposal
# distributions and the logspace acceptance, random draws from torch's
# generator seeded before each call.
MGEN = {"nwalkers": 16, "nelec": 2, "ndim": 3, "nstep": 24, "step_size": 0.4,
        "ntherm": -8, "ndecor": 2, "seed": 4040}
MGEN_CASES = (("all-elec", "normal", False), ("one-elec", "uniform", False),
              ("all-elec-iter", "normal", False), ("all-elec", "normal", True),
              ("one-elec", "normal", False), ("all-elec-iter", "uniform", True))


def make_metropolis_generic(reference_root):
    ref_stubs.install(reference_root)
    import torch
    from qmctorch.sampler import Metropolis
    from qmctorch.utils import set_torch_double_precision

    set_torch_double_precision()
    a, c = gmet_density_params()
    at, ct = torch.as_tensor(a), torch.as_tensor(c)

    def pdf(x):
        return torch.exp(-(at * (x - ct) ** 2).sum(-1))

    g = MGEN
    pos0 = np.random.default_rng(8).normal(size=(g["nwalkers"], g["nelec"] * g["ndim"]))
    out = {"pos0": pos0}
    for i, (mtype, proba, logspace) in enumerate(MGEN_CASES):
        sampler = Metropolis(nwalkers=g["nwalkers"], nstep=g["nstep"], step_size=g["step_size"],
                             ntherm=g["ntherm"], ndecor=g["ndecor"], nelec=g["nelec"],
                             ndim=g["ndim"], init={"method": "uniform", "min": -1, "max": 1},
                             move={"type": mtype, "proba": proba}, logspace=logspace)
        torch.manual_seed(g["seed"] + i)
        samples = sampler(pdf, pos=torch.as_tensor(pos0).clone(), with_tqdm=False)
        out["samples_%d" % i] = samples.detach().numpy()
        out["final_%d" % i] = sampler.walkers.pos.detach().numpy()
    out_file = os.path.join(HERE, "metropolis_generic.npz")
    np.savez_compressed(out_file, **out)
    print("wrote", out_file, os.path.getsize(out_file), "bytes")


# Chains of the reference HMC sampler (hamiltonian.py:10-201): on the analytic
# density of the drift-diffusion fixture, and on the H2 sto-3g SlaterJastrow of
# the "h2" case (forces by the reference's autograd through the density).
HMC = {"nwalkers": 16, "nelec": 2, "ndim": 3, "nstep": 12, "step_size": 0.1, "L": 6,
       "ntherm": -6, "ndecor": 2, "seed": 777}


def make_hamiltonian(reference_root):
    ref_stubs.install(reference_root)
    import torch
    from qmctorch.sampler.hamiltonian import Hamiltonian
    from qmctorch.utils import set_torch_double_precision
    from qmctorch.wavefunction import SlaterJastrow
    from qmctorch_gb300.scf import Molecule

    set_torch_double_precision()
    a, c = gmet_density_params()
    at, ct = torch.as_tensor(a), torch.as_tensor(c)

    def pdf(x):
        return torch.exp(-(at * (x - ct) ** 2).sum(-1))

    g = HMC
    pos0 = np.random.default_rng(9).normal(size=(g["nwalkers"], g["nelec"] * g["ndim"]))

    def sampler():
        return Hamiltonian(nwalkers=g["nwalkers"], nstep=g["nstep"], step_size=g["step_size"],
                           L=g["L"], ntherm=g["ntherm"], ndecor=g["ndecor"], nelec=g["nelec"],
                           ndim=g["ndim"], init={"method": "uniform", "min": -1, "max": 1})
    s = sampler()
    torch.manual_seed(g["seed"])
    samples = s(pdf, pos=torch.as_tensor(pos0), with_tqdm=False)
    atoms, unit, basis, configs, all_mo = CASES["h2"][:5]
    torch.manual_seed(1234)
    mol = Molecule(atoms, unit=unit, basis=basis, calculator="huckel")
    wf = SlaterJastrow(mol, configs=configs, include_all_mo=all_mo)
    h2pos0 = seeded_positions(mol, g["nwalkers"], seed=31)
    s2 = sampler()
    torch.manual_seed(g["seed"] + 1)
    h2samples = s2(wf.pdf, pos=torch.as_tensor(h2pos0), with_tqdm=False)
    out_file = os.path.join(HERE, "hamiltonian.npz")
    np.savez_compressed(out_file, pos0=pos0, samples=samples.detach().numpy(),
                        h2_pos0=h2pos0, h2_samples=h2samples.detach().numpy(),
                        **{"cfg_" + k: np.asarray(v) for k, v in HMC.items()})
    print("wrote", out_file, os.path.getsize(out_file), "bytes")


# The reference's single-precision run (set_torch_single_precision,
# utils/torch_utils.py:16-21) of the LiH cas(2,2) case: psi, E_L and the
# manual / automatic parameter gradients of its FP32 autograd.
def make_fp32(reference_root):
    ref_stubs.install(reference_root)
    import torch
    from qmctorch.sampler import Metropolis
    from qmctorch.solver import Solver
    from qmctorch.utils.torch_utils import set_torch_single_precision
    from qmctorch.wavefunction import SlaterJastrow
    from qmctorch_gb300.scf import Molecule

    atoms, unit, basis, configs, all_mo, nw = CASES["lih_cas"][:6]
    torch.manual_seed(1234)
    mol = Molecule(atoms, unit=unit, basis=basis, calculator="huckel")
    set_torch_single_precision()
    try:
        wf = SlaterJastrow(mol, configs=configs, include_all_mo=all_mo)
        g = torch.Generator().manual_seed(7)
        wf.fc.weight.data = torch.rand(wf.fc.weight.shape, generator=g).float()
        pos = torch.as_tensor(seeded_positions(mol, nw, seed=11), dtype=torch.float32)
        data = {"pos32": pos.numpy(), "fc_weight32": wf.fc.weight.detach().numpy().reshape(-1)}
        with torch.no_grad():
            data.update(psi32=wf(pos).numpy(), eloc32=wf.local_energy(pos).numpy())
        sampler = Metropolis(nwalkers=nw, nstep=2, step_size=0.2, nelec=mol.nelec,
                             init=mol.domain("atomic"))
        opt = torch.optim.Adam(wf.parameters(), lr=1e-3)
        solver = Solver(wf=wf, sampler=sampler, optimizer=opt, output="_unused.hdf5")
        names = ["ao.bas_exp", "mo.mo_modifier", "jastrow.jastrow_kernel.weight", "fc.weight"]
        params = dict(wf.named_parameters())
        for mode in ("manual", "auto"):
            solver.configure(grad=mode, loss="energy", track=["local_energy"])
            solver.loss.use_weight = False
            opt.zero_grad()
            wf.zero_grad()
            loss, _ = solver.evaluate_gradient(pos.clone().requires_grad_(mode == "auto"))
            data["grad32_%s_loss" % mode] = np.asarray(float(loss))
            for n in names:
                gr = params[n].grad
                data["grad32_%s_%s" % (mode, n)] = (np.zeros(params[n].shape) if gr is None
                                                    else gr.detach().numpy().copy())
    finally:
        torch.set_default_dtype(torch.float64)
    out_file = os.path.join(HERE, "lih_cas_fp32.npz")
    np.savez_compressed(out_file, **data)
    print("wrote", out_file, os.path.getsize(out_file), "bytes")


EXTRA = {"gmetropolis": "make_gmetropolis", "walkers": "make_walkers", "fp32": "make_fp32",
         "metropolis_generic": "make_metropolis_generic", "hamiltonian": "make_hamiltonian"}


if __name__ == "__main__":
    args = sys.argv[1:]
    root = os.environ.get("QMCTORCH_REFERENCE")
    if root is None:
        if not args:
            sys.exit("usage: make_golden.py REFERENCE_ROOT [case ...] "
                     "(or set QMCTORCH_REFERENCE)")
        root, args = args[0], args[1:]
    names = tuple(args)
    for extra, fn in EXTRA.items():
        if extra in names or not names:
            globals()[fn](root)
    names = tuple(n for n in names if n not in EXTRA)
    if names or not args:
        main(root, names)
