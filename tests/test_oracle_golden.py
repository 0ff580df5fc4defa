"""Pin the CPU oracle to the reference: every oracle output is compared with
the golden vectors the reference package produced on the same inputs."""
import numpy as np
import pytest

from oracle import qmc_oracle as orc
from tests.golden_cases import CASES, EN_CASES, STO_CASES, jastrow_weights, load

ALL = CASES + EN_CASES + STO_CASES

RTOL = 1e-10


def _oracle(mol, d):
    return orc.OracleSlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"],
                                   jastrow_terms=jastrow_weights(d), fc_weight=d["fc_weight"])


def close(a, b, rtol=RTOL, atol_scale=1e-12):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    atol = atol_scale * max(1.0, float(np.abs(b).max()))
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


@pytest.mark.parametrize("name", ALL)
def test_oracle_wavefunction(name):
    mol, d = load(name)
    wf = _oracle(mol, d)
    pos = d["pos"]
    if "ao" in d:
        ao, dao, d2ao = orc.ao_values(wf.basis, pos, [0, 1, 2])
        close(ao, d["ao"])
        close(dao, d["dao"])
        close(d2ao, d["d2ao"])
        close(orc.ao_values(wf.basis, pos, 1), d["ao_sumgrad"])
        close(ao @ wf.W, d["mo"])
        j, dj, d2j = wf.jastrow(pos, [0, 1, 2], sum_grad=False)
        close(j, d["jast"])
        close(dj, d["djast"])
        close(d2j, d["d2jast"])
        close(wf.jastrow(pos, 1), d["djast_sum"])
        close(wf.pool.dets(ao @ wf.W), d["dets"], rtol=1e-9)
    close(wf.forward(pos), d["psi"], rtol=1e-9)
    close(wf.pdf(pos), d["pdf"], rtol=1e-9)
    close(wf.kinetic_energy(pos), d["kinetic"], rtol=1e-9)
    close(wf.local_energy(pos), d["eloc"], rtol=1e-9)
    close(wf.nuclear_potential(pos), d["v_en"])
    close(wf.electronic_potential(pos), d["v_ee"])
    close(wf.nuclear_repulsion(), d["v_nn"])


@pytest.mark.parametrize("name", [c for c in ALL if "met_out" in load(c)[1]])
def test_oracle_metropolis_replay(name):
    mol, d = load(name)
    wf = _oracle(mol, d)
    out, nacc, _ = orc.metropolis_replay(wf.pdf, d["met_pos0"], d["met_props"], d["met_unif"],
                                         ntherm=int(d["met_ntherm"]), ndecor=int(d["met_ndecor"]))
    close(out, d["met_out"])


@pytest.mark.parametrize("name", [c for c in ALL if "iter_out" in load(c)[1]])
def test_oracle_metropolis_iter_replay(name):
    mol, d = load(name)
    wf = _oracle(mol, d)
    out, _, _ = orc.metropolis_replay(wf.pdf, d["iter_pos0"], d["iter_props"], d["iter_unif"],
                                      move_type="all-elec-iter")
    close(out, d["iter_out"])


@pytest.mark.parametrize("name", [c for c in ALL if "one_out" in load(c)[1]])
def test_oracle_metropolis_one_elec_replay(name):
    """one-elec moves: the electron index each walker moves per step was drawn
    by the reference (torch.LongTensor.random_, metropolis.py:247) and is
    replayed with its proposals and uniforms."""
    mol, d = load(name)
    wf = _oracle(mol, d)
    nstep, nw = d["one_unif"].shape
    out, _, _ = orc.metropolis_replay(wf.pdf, d["one_pos0"], d["one_props"][:, None],
                                      d["one_unif"][:, None], ntherm=int(d["one_ntherm"]),
                                      ndecor=int(d["one_ndecor"]), move_type="one-elec",
                                      electron_index=d["one_index"][:, None])
    close(out, d["one_out"])


def test_configs_match_reference_counts():
    mol, d = load("h2o_sd")
    cu, cd = orc.get_configs("single_double(4,4)", 5, 5, 24)
    assert len(cu) == 27 and int(max(cu.max(), cd.max())) + 1 == 7
    cu, cd = orc.get_configs("cas(2,2)", 2, 2, 6)
    assert cu.tolist() == [[0, 1], [0, 1], [0, 2], [0, 2]]
