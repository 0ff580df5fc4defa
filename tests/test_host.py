"""CPU tests: the C ABI library loads and exports what the header declares,
and the host-side table builders agree with the oracle's restatement of the
reference index logic."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

from oracle import qmc_oracle as orc
from qmctorch_gb300 import _lib
from qmctorch_gb300.scf import Molecule
from qmctorch_gb300.wavefunction import SlaterJastrow
from qmctorch_gb300.wavefunction.tables import BasisTables, ConfigTables, OrbitalConfigurations
from tests.golden_cases import CASES, load

HEADER = os.path.join(_lib.ROOT, "include", "qmc_gb300.h")
INCLUDE = os.path.join(_lib.ROOT, "include")


def header_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        src = open(os.path.join(INCLUDE, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(qmc_\w+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_header_symbol():
    lib = _lib.lib()
    names = header_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, n
    assert lib.qmc_version().startswith(b"qmc_gb300")


def test_struct_layout_matches_header_order():
    src = open(HEADER).read()
    body = src[src.index("typedef struct qmc_wf_desc"):src.index("} qmc_wf_desc;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";")[:-1]:
        decl = decl.split("{")[-1]
        for part in decl.split(","):
            m = re.search(r"(\w+)\s*(\[\d\])?\s*$", part.strip())
            if m:
                fields.append(m.group(1))
    assert fields == [f[0] for f in _lib.WfDesc._fields_]


def _desc_for(name):
    mol, d = load(name)
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"])
    keep = []

    def p(t):
        t = t.detach().contiguous()
        keep.append(t)
        return ctypes.c_void_p(t.data_ptr())

    desc = _lib.WfDesc()
    bt, ct = wf.ao._tables, wf.pool._tables
    desc.nelec, desc.nup, desc.ndown = mol.nelec, mol.nup, mol.ndown
    desc.natom, desc.nao, desc.nmo = mol.natom, mol.basis.nao, wf.mo.mo_scf.shape[1]
    desc.nmo_used = wf.highest_occ_mo
    desc.ngroup, desc.ngprim, desc.nweight, desc.contract = bt.ngroup, bt.ngprim, bt.nweight, 1
    desc.use_jastrow = 1
    for f in ("atom_coords", "atom_charge", "bas_exp", "mo_scf", "mo_modifier", "jastrow_w",
              "ci_weight"):
        setattr(desc, f, p(torch.ones(4)))
    for f in ("group_atom", "group_prim", "group_ao", "gprim_entry", "ao_k", "ao_wofs"):
        setattr(desc, f, p(bt.t[f]))
    desc.ao_wd = p(bt.t["ao_wd"])
    desc.weight_entry = p(bt.t["w_entry"])
    desc.det_mode = int(ct.explicit)
    desc.ncfg = ct.ncfg
    desc.max_orb[0], desc.max_orb[1] = ct.max_orb
    desc.ndet[0], desc.ndet[1] = ct.ndet
    desc.det_table[0], desc.det_table[1] = p(ct.t["det_table0"]), p(ct.t["det_table1"])
    desc.cfg_det[0], desc.cfg_det[1] = p(ct.t["cfg_det0"]), p(ct.t["cfg_det1"])
    return desc, keep, wf


@pytest.mark.parametrize("name", CASES)
def test_scratch_sizes_and_argument_checks(name):
    lib = _lib.lib()
    desc, keep, wf = _desc_for(name)
    b0 = lib.qmc_scratch_bytes(ctypes.byref(desc), 1000, 0)
    b1 = lib.qmc_scratch_bytes(ctypes.byref(desc), 1000, 1)
    bm = lib.qmc_metropolis_scratch_bytes(ctypes.byref(desc), 1000)
    assert 0 < b0 < b1 and b0 <= bm
    assert b0 % (8 * 1024) == 0  # 1000 walkers padded to 1024 slots
    # argument errors are reported, never launched (no GPU needed)
    assert lib.qmc_wf_psi(ctypes.byref(desc), None, 10, None, None, 0, None) == 1
    assert lib.qmc_wf_psi(ctypes.byref(desc), ctypes.c_void_p(8), 10, ctypes.c_void_p(8),
                          ctypes.c_void_p(8), 8, None) == 3
    assert lib.qmc_wf_psi(None, None, 0, None, None, 0, None) == 1
    desc.nup = 100
    desc.nelec = 100 + desc.ndown
    assert lib.qmc_wf_psi(ctypes.byref(desc), None, 0, None, None, 0, None) == 2
    assert lib.qmc_status_string(3) == b"scratch buffer too small"


@pytest.mark.parametrize("name", CASES)
def test_config_tables_match_oracle(name):
    mol, d = load(name)
    oc = OrbitalConfigurations(mol).get_configs(d["configs"])
    cu, cd = orc.get_configs(d["configs"], mol.nup, mol.ndown, mol.basis.nmo)
    assert np.array_equal(oc[0].numpy(), cu) and np.array_equal(oc[1].numpy(), cd)
    ct = ConfigTables(d["configs"], oc, mol.nup, mol.ndown)
    op = orc.OraclePool(d["configs"], (cu, cd), mol.nup, mol.ndown)
    if op.explicit:
        assert np.array_equal(ct.t["det_table0"].numpy().reshape(-1, mol.nup), op.ucfg_up)
        assert np.array_equal(ct.t["cfg_det0"].numpy(), op.iucfg_up)
        assert np.array_equal(ct.t["cfg_det1"].numpy(), op.iucfg_dn)
    else:
        tab = ct.t["det_table0"].numpy().reshape(-1, 5)
        assert [int(r[1]) for r in tab if r[0] == 1] == op.single_up
        assert [int(x) for r in tab if r[0] == 2 for x in r[1:]] == op.double_up
        tab = ct.t["det_table1"].numpy().reshape(-1, 5)
        assert [int(r[1]) for r in tab if r[0] == 1] == op.single_dn
        assert np.array_equal(ct.t["cfg_det0"].numpy(), op.index_unique_exc[0])
        assert np.array_equal(ct.t["cfg_det1"].numpy(), op.index_unique_exc[1])


def test_basis_groups_share_exponents():
    mol, _ = load("h2o_sd")
    bt = BasisTables(mol.basis, mol.basis.bas_exp)
    assert bt.nweight == len(mol.basis.bas_exp) == 56
    assert bt.ngprim == 28 and bt.ngroup == 11
    ga = bt.t["group_ao"].numpy()
    assert ga[-1] == mol.basis.nao and np.all(np.diff(ga) <= 6)
    # training that splits a group regroups
    e = np.array(mol.basis.bas_exp, dtype=np.float64)
    e[-1] *= 1.01  # last d component of the last atom group
    assert not bt.still_valid(e)
    bt2 = BasisTables(mol.basis, e)
    assert bt2.ngroup > bt.ngroup


def test_molecule_roundtrip(tmp_path):
    mol = Molecule("Li 0 0 0; H 0 0 1.595", unit="angs", basis="sto-3g")
    f = str(tmp_path / "lih.npz")
    mol.save(f)
    m2 = Molecule(load=f)
    assert m2.nelec == 4 and m2.nup == 2 and m2.basis.nao == 6
    assert np.allclose(m2.basis.mos, mol.basis.mos)
    assert mol.domain("atomic")["atom_nelec"] == [3, 1]


def test_missing_gpu_fails_loudly():
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    mol, d = load("h2")
    wf = SlaterJastrow(mol)
    with pytest.raises(RuntimeError, match="CUDA"):
        wf(torch.zeros(2, 6))


@pytest.mark.parametrize("name", ["h2o_sd", "lih_cas"])
def test_new_entry_points_reject_bad_arguments_without_a_gpu(name):
    """Batch Metropolis, statistics, position gradients and the local-energy
    adjoint report argument errors before touching the device."""
    lib = _lib.lib()
    desc, keep, wf = _desc_for(name)
    args = (_lib.MetropolisArgs * 2)()
    descs = (_lib.WfDesc * 2)(desc, desc)
    scr = (ctypes.c_void_p * 2)(ctypes.c_void_p(8), ctypes.c_void_p(8))
    nb = (ctypes.c_int64 * 2)(1 << 40, 1 << 40)
    assert lib.qmc_metropolis_run_batch(descs, args, scr, nb, 0, None) == 1
    assert lib.qmc_metropolis_run_batch(descs, args, scr, nb, 33, None) == 1
    for a in args:
        a.nwalkers, a.nstep, a.ndecor, a.pos = 4, 1, 1, ctypes.c_void_p(8)
    args[1].move_type = 2  # single-electron moves are not batched
    assert lib.qmc_metropolis_run_batch(descs, args, scr, nb, 2, None) == 5
    args[1].move_type = 0
    descs[1].precision = 1 - descs[0].precision
    assert lib.qmc_metropolis_run_batch(descs, args, scr, nb, 2, None) == 2
    assert lib.qmc_reduce_stats(ctypes.c_void_p(8), 0, ctypes.c_void_p(8), ctypes.c_void_p(8), 64,
                                None) == 1
    assert lib.qmc_reduce_stats(ctypes.c_void_p(8), 10 ** 6, ctypes.c_void_p(8),
                                ctypes.c_void_p(8), 8, None) == 3
    assert lib.qmc_reduce_scratch_bytes(10 ** 6) > lib.qmc_reduce_scratch_bytes(10)
    assert lib.qmc_wf_gradients(ctypes.byref(desc), None, -1, 0, None, None, 0, None) == 1
    assert lib.qmc_wf_gradients(ctypes.byref(desc), ctypes.c_void_p(8), 10, 0, ctypes.c_void_p(8),
                                ctypes.c_void_p(8), 8, None) == 3
    # launch-plan diagnostics: argument errors before the occupancy query
    assert lib.qmc_metropolis_plan(ctypes.byref(desc), 16, None) == 1
    assert lib.qmc_metropolis_plan(ctypes.byref(desc), 0, (ctypes.c_int32 * 5)()) == 1
    # the Metropolis scratch holds the walkers' positions too (split coordinates)
    per = 3 * desc.nelec * (8 if desc.precision == 1 else 16)
    assert (lib.qmc_metropolis_scratch_bytes(ctypes.byref(desc), 1024)
            - lib.qmc_scratch_bytes(ctypes.byref(desc), 1024, 0)) >= per * 1024
    gb = lib.qmc_eloc_adjoint_scratch_bytes(ctypes.byref(desc), 100)
    assert gb > lib.qmc_adjoint_scratch_bytes(ctypes.byref(desc), 100) > 0
    v = ctypes.c_void_p(8)
    assert lib.qmc_wf_local_energy_adjoint(ctypes.byref(desc), v, 10, v, v, 1, v, v, 0, v, v, v,
                                           gb, None) == 1  # ldw < nmo_used
    assert lib.qmc_wf_local_energy_adjoint(ctypes.byref(desc), v, 10, v, v, 1, v, v,
                                           desc.nmo_used, v, v, v, 8, None) == 3


def test_tensor_core_mo_rejects_bad_arguments_and_shapes_without_a_gpu():
    """qmc_mo_eval_tc checks arguments and its shape limits (nmo <= 256, the
    split operand tiles within 227 KB of shared memory) before any device
    call; an empty batch is a no-op."""
    lib = _lib.lib()
    desc, keep, wf = _desc_for("h2o_sd")
    v = ctypes.c_void_p(8)
    assert lib.qmc_mo_eval_tc(None, v, 10, v, None) == 1
    assert lib.qmc_mo_eval_tc(ctypes.byref(desc), v, -1, v, None) == 1
    assert lib.qmc_mo_eval_tc(ctypes.byref(desc), None, 10, v, None) == 1
    assert lib.qmc_mo_eval_tc(ctypes.byref(desc), None, 0, None, None) == 0
    desc.nmo = 300
    assert lib.qmc_mo_eval_tc(ctypes.byref(desc), v, 10, v, None) == 2
    desc.nmo, desc.nao = 128, 200
    assert lib.qmc_mo_eval_tc(ctypes.byref(desc), v, 10, v, None) == 2
    mol, d = load("h2")
    old = torch.get_default_dtype()
    try:
        torch.set_default_dtype(torch.float32)
        assert SlaterJastrow(mol).mo.precision == "mixed"
        assert SlaterJastrow(mol, precision="fp64").mo.precision == "fp64"
        torch.set_default_dtype(torch.float64)
        assert SlaterJastrow(mol).mo.precision == "fp64"
        assert SlaterJastrow(mol, precision="mixed").mo.precision == "mixed"
    finally:
        torch.set_default_dtype(old)


def test_pipeline_wait_limit_is_host_settable_without_a_gpu():
    """qmc_set_wait_limit_ns stores the limit of the tensor-core kernel's
    pipeline waits for later launches and returns the previous one."""
    lib = _lib.lib()
    old = lib.qmc_set_wait_limit_ns(12345)
    try:
        assert old == 1000000000
        assert lib.qmc_set_wait_limit_ns(0) == 12345
    finally:
        lib.qmc_set_wait_limit_ns(old)
    assert lib.qmc_status_string(7).startswith(b"a bounded pipeline wait")


def test_descriptor_is_reused_only_while_its_sources_keep_their_values():
    """SlaterJastrow._desc returns the descriptor it built last while every
    tensor it was built from is the same object with the same values, and
    builds a new one after any change, including writes through ``.data``
    (which leave a tensor's version counter alone)."""
    mol = Molecule("H 0 0 0; H 0 0 0.74", unit="angs", basis="sto-3g", calculator="huckel")
    wf = SlaterJastrow(mol, configs="single_double(2,2)")
    dev = torch.device("cpu")
    c1 = wf._desc(dev)
    assert wf._desc(dev) is c1
    wf.fc.weight.data[0][1] = 0.25  # no version change
    c2 = wf._desc(dev)
    assert c2 is not c1
    w = ctypes.cast(c2.desc.ci_weight, ctypes.POINTER(ctypes.c_double))
    assert w[1] == 0.25
    with torch.no_grad():
        wf.jastrow.jastrow_kernel.weight.add_(0.5)
    c3 = wf._desc(dev)
    assert c3 is not c2
    jw = ctypes.cast(c3.desc.jastrow_w, ctypes.POINTER(ctypes.c_double))
    assert jw[0] == float(wf.jastrow.jastrow_kernel.weight.detach())
    wf.mo.mo_scf = torch.nn.Parameter(wf.mo.mo_scf.detach().clone() * 2.0)
    c4 = wf._desc(dev)
    assert c4 is not c3
    assert wf._desc(dev) is c4
    wf.ao.atom_coords.data[1, 2] += 0.1  # geometry: V_nn follows
    c5 = wf._desc(dev)
    assert c5 is not c4 and c5.desc.e_nuc != c4.desc.e_nuc


@pytest.mark.parametrize("name", ["h2o_sd", "lih_cas"])
def test_drift_sampler_rejects_bad_arguments_without_a_gpu(name):
    """qmc_drift_run checks its arguments (step, decorrelation, replay inputs
    all or none, snapshot buffer, scratch size) before any device call; an
    empty run is a no-op."""
    lib = _lib.lib()
    desc, keep, wf = _desc_for(name)
    v = ctypes.c_void_p(8)
    a = _lib.DriftArgs()
    a.pos, a.nwalkers, a.nstep, a.ntherm, a.ndecor, a.step_size = v, 16, 4, 0, 1, 0.2
    need = lib.qmc_drift_scratch_bytes(ctypes.byref(desc), 16)
    assert need > 0 and lib.qmc_drift_scratch_bytes(ctypes.byref(desc), 1024) > need
    assert lib.qmc_drift_run(ctypes.byref(desc), None, v, need, None) == 1
    assert lib.qmc_drift_run(ctypes.byref(desc), ctypes.byref(a), v, need - 8, None) == 3
    a.step_size = 0.0
    assert lib.qmc_drift_run(ctypes.byref(desc), ctypes.byref(a), v, need, None) == 1
    a.step_size, a.ndecor = 0.2, 0
    assert lib.qmc_drift_run(ctypes.byref(desc), ctypes.byref(a), v, need, None) == 1
    a.ndecor, a.normals = 1, v  # replay needs all three inputs
    assert lib.qmc_drift_run(ctypes.byref(desc), ctypes.byref(a), v, need, None) == 1
    a.normals, a.nsnap = None, 2  # snapshots without a buffer
    assert lib.qmc_drift_run(ctypes.byref(desc), ctypes.byref(a), v, need, None) == 1
    a.nsnap, a.nstep = 0, 0
    assert lib.qmc_drift_run(ctypes.byref(desc), ctypes.byref(a), None, 0, None) == 0


def test_hmc_sampler_rejects_bad_arguments_without_a_gpu():
    """qmc_hmc_run checks its arguments (step, trajectory length, decorrelation,
    replay inputs both or none, snapshot buffer, scratch size) before any
    device call; an empty run is a no-op."""
    lib = _lib.lib()
    desc, keep, wf = _desc_for("h2o_sd")
    v = ctypes.c_void_p(8)
    a = _lib.HmcArgs()
    a.pos, a.nwalkers, a.nstep, a.ntherm, a.ndecor = v, 16, 4, 0, 1
    a.traj_length, a.step_size = 5, 0.1
    need = lib.qmc_hmc_scratch_bytes(ctypes.byref(desc), 16)
    assert need > 0
    assert lib.qmc_hmc_run(ctypes.byref(desc), None, v, need, None) == 1
    assert lib.qmc_hmc_run(ctypes.byref(desc), ctypes.byref(a), v, need - 8, None) == 3
    a.traj_length = 0
    assert lib.qmc_hmc_run(ctypes.byref(desc), ctypes.byref(a), v, need, None) == 1
    a.traj_length, a.step_size = 5, -0.1
    assert lib.qmc_hmc_run(ctypes.byref(desc), ctypes.byref(a), v, need, None) == 1
    a.step_size, a.momenta = 0.1, v  # replay needs both inputs
    assert lib.qmc_hmc_run(ctypes.byref(desc), ctypes.byref(a), v, need, None) == 1
    a.momenta, a.nsnap = None, 3  # snapshots without a buffer
    assert lib.qmc_hmc_run(ctypes.byref(desc), ctypes.byref(a), v, need, None) == 1
    a.nsnap, a.nstep = 0, 0
    assert lib.qmc_hmc_run(ctypes.byref(desc), ctypes.byref(a), None, 0, None) == 0
