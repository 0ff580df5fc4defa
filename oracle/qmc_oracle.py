"""CPU oracle for the QMCTorch VMC hot path -- TEST INFRASTRUCTURE ONLY.

This module restates, in FP64 numpy, the reference's algorithm for the path
``SlaterJastrow.forward / pdf / local_energy`` and ``Metropolis`` sampling.
It is the checker for the CUDA implementation: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it. The product path never calls it.

Parity pin: every function is checked against golden vectors produced by
running the reference package itself (``tests/golden/make_golden.py``), see
``tests/test_oracle_golden.py``.

Each function cites the reference lines it restates (paths relative to the
QMCTorch repository).
"""
from __future__ import annotations

import numpy as np

DF = {-1: 1, 0: 1, 1: 1, 2: 2, 3: 3, 5: 15}


# ----------------------------------------------------------------------------
# basis / AO layer
# ----------------------------------------------------------------------------
class OracleBasis:
    """Flat basis tables read from a basis namespace
    (``qmctorch/wavefunction/orbitals/atomic_orbitals.py:15-102``)."""

    def __init__(self, basis, atom_coords, bas_exp=None):
        self.nao = int(basis.nao)
        self.atom_coords = np.asarray(atom_coords, dtype=np.float64)
        self.nshells = np.asarray(basis.nshells)
        self.index_ctr = np.asarray(basis.index_ctr)
        self.contract = len(np.unique(self.index_ctr)) != len(self.index_ctr)
        self.bas_coeffs = np.asarray(basis.bas_coeffs, dtype=np.float64)
        self.bas_exp = np.asarray(basis.bas_exp if bas_exp is None else bas_exp, dtype=np.float64)
        self.k = np.stack([np.asarray(basis.bas_kx), np.asarray(basis.bas_ky),
                           np.asarray(basis.bas_kz)], axis=1).astype(np.int64)
        self.radial = str(getattr(basis, "radial_type", "gto_pure"))
        self.kr = np.asarray(getattr(basis, "bas_kr", np.zeros(len(self.bas_exp))),
                             dtype=np.float64)
        # norm_orbital.py:136-161, computed from the namespace exponents once
        # (atomic_orbitals.py:93-94)
        a = np.asarray(basis.bas_exp, dtype=np.float64)
        norm = (2.0 * a / np.pi) ** 0.75
        for d in range(3):
            kd = self.k[:, d]
            df = np.array([DF[int(2 * v - 1)] for v in kd], dtype=np.float64)
            norm = norm * (4.0 * a) ** (kd / 2.0) / np.sqrt(df)
        self.norm_cst = norm
        if self.radial.startswith("sto"):
            # norm_slater_cartesian (norm_orbital.py:106-161)
            kk = self.k
            lv = kk.sum(1) + self.kr + 1.0
            lfact = np.array([float(np.prod(np.arange(1, int(2 * v) + 1))) for v in lv])
            pref = 4.0 * np.pi * lfact / (2.0 * a) ** (2.0 * lv + 1.0)
            num = np.prod(np.array([[DF[int(2 * v - 1)] for v in row] for row in kk],
                                   dtype=np.float64), axis=1)
            den = np.array([DF[int(2 * s_ + 1)] for s_ in kk.sum(1)], dtype=np.float64)
            self.norm_cst = np.sqrt(1.0 / (pref * num / den))
        # index_add of the contraction (atomic_orbitals.py:654-669) as a
        # (primitive x AO) matrix of the bas_coeffs
        self.contraction = np.zeros((len(self.index_ctr), self.nao))
        self.contraction[np.arange(len(self.index_ctr)), self.index_ctr] = self.bas_coeffs


def _fast_power(x, k):
    """x**k for k in {0,1,2} (``qmctorch/utils/torch_utils.py:24-59``)."""
    out = np.where(k == 0, 1.0, x)
    return np.where(k == 2, out * out, out)


def _index_add(nb, ne, nao, idx, vals, extra=()):
    out = np.zeros((nb, ne, nao) + tuple(extra))
    # index_add over axis 2
    np.add.at(out, (slice(None), slice(None), idx), vals)
    return out


def ao_values(b: OracleBasis, pos, derivative=0, sum_grad=True):
    """AO values / gradients / laplacians
    (``atomic_orbitals.py:131-218, 220-249, 290-356, 397-423, 578-669``;
    ``radial_functions.py:241-320``; ``spherical_harmonics.py:102-199``).

    derivative: 0 -> (nb,ne,nao); 1 -> (nb,ne,nao,3) if not sum_grad else (nb,ne,nao);
    2 -> (nb,ne,nao) laplacian; [0,1,2] -> (ao, dao (grad), d2ao).
    """
    pos = np.asarray(pos, dtype=np.float64)
    nb = pos.shape[0]
    ne = pos.shape[1] // 3
    # _elec_atom_dist 633-652 + _process_position 611-631
    xyz = pos.reshape(nb, ne, 1, 3) - b.atom_coords[None, None]
    r = np.sqrt((xyz * xyz).sum(3))
    xyz = np.repeat(xyz, b.nshells, axis=2)
    r = np.repeat(r, b.nshells, axis=2)
    alpha = b.bas_exp
    if b.radial.startswith("sto"):
        return _sto_ao_values(b, xyz, r, derivative, sum_grad, nb, ne)
    # radial_gaussian_pure
    R2 = r * r
    er = np.exp(-alpha * R2)
    # cartesian harmonics
    k = b.k
    xyz_k = _fast_power(xyz, k)
    Y = xyz_k.prod(-1)
    nc = b.norm_cst
    cc = b.bas_coeffs
    idx = b.index_ctr

    def derivs():  # radial and harmonic derivative pieces (only when asked for)
        bexp_er = alpha * er
        nabla_er = -2.0 * bexp_er[..., None] * xyz          # (nb,ne,np,3)
        lap_er = alpha * er * (4.0 * alpha * R2 - 6.0)      # sum_hess
        km1 = np.maximum(k - 1, 0)
        km2 = np.maximum(k - 2, 0)
        xyz_km1 = _fast_power(xyz, km1)
        xyz_km2 = _fast_power(xyz, km2)
        kx, ky, kz = k[:, 0], k[:, 1], k[:, 2]
        dY = np.stack((kx * xyz_km1[..., 0] * xyz_k[..., 1] * xyz_k[..., 2],
                       ky * xyz_k[..., 0] * xyz_km1[..., 1] * xyz_k[..., 2],
                       kz * xyz_k[..., 0] * xyz_k[..., 1] * xyz_km1[..., 2]), axis=-1)
        d2Y = (kx * (kx - 1) * xyz_km2[..., 0] * xyz_k[..., 1] * xyz_k[..., 2]
               + ky * (ky - 1) * xyz_k[..., 0] * xyz_km2[..., 1] * xyz_k[..., 2]
               + kz * (kz - 1) * xyz_k[..., 0] * xyz_k[..., 1] * xyz_km2[..., 2])
        return nabla_er, lap_er, dY, d2Y

    def contract(v):  # _contract 654-669 (value path applies coeffs only here)
        if b.contract:
            return v @ b.contraction
        return v

    def ao_kernel():  # _ao_kernel 236-249
        return contract(nc * er * Y)

    def grad_kernel(nabla_er, dY):  # _gradient_kernel 330-356
        bas = nabla_er * Y[..., None] + er[..., None] * dY
        bas = nc[:, None] * cc[:, None] * bas
        if b.contract:
            return _index_add(nb, ne, b.nao, idx, bas, extra=(3,))
        return bas

    def sum_grad_kernel(nabla_er, dY):  # _sum_gradient_kernel 290-307
        dR = nabla_er.sum(3)
        dYs = dY.sum(-1)
        return contract(nc * (dR * Y + er * dYs))

    def lap_kernel(nabla_er, lap_er, dY, d2Y):  # _sum_diag_hessian_kernel 397-423
        return contract(nc * (lap_er * Y + 2.0 * (nabla_er * dY).sum(3) + er * d2Y))

    if derivative == 0 or derivative == [0]:
        return ao_kernel()
    nabla_er, lap_er, dY, d2Y = derivs()
    if derivative == 1 or derivative == [1]:
        return sum_grad_kernel(nabla_er, dY) if sum_grad else grad_kernel(nabla_er, dY)
    if derivative == 2 or derivative == [2]:
        return lap_kernel(nabla_er, lap_er, dY, d2Y)
    if list(derivative) == [0, 1, 2]:
        return ao_kernel(), grad_kernel(nabla_er, dY), lap_kernel(nabla_er, lap_er, dY, d2Y)
    raise ValueError("derivative must be 0, 1, 2 or [0, 1, 2]")


def _sto_ao_values(b, xyz, r, derivative, sum_grad, nb, ne):
    """Slater-type AOs (radial_slater / radial_slater_pure,
    radial_functions.py:6-123, 323-406) times cartesian harmonics, combined
    as atomic_orbitals.py:236-423 combines radial and angular parts; the ADF
    layout is uncontracted (one entry per AO, coefficients 1)."""
    alpha = b.bas_exp
    n = b.kr if b.radial == "sto" else np.zeros_like(b.kr)
    k = b.k
    er = np.exp(-alpha * r)
    rn = r ** n
    R = rn * er
    xyz_k = _fast_power(xyz, k)
    Y = xyz_k.prod(-1)
    nc = b.norm_cst
    if derivative == 0 or derivative == [0]:
        return nc * R * Y
    nrm2 = n * r ** (n - 2)
    nabla_rn = nrm2[..., None] * xyz
    nabla_er = -(alpha * er)[..., None] * xyz / r[..., None]
    nabla_R = nabla_rn * er[..., None] + rn[..., None] * nabla_er
    lap_R = (nrm2 * (n + 1)) * er + 2.0 * (nabla_rn * nabla_er).sum(-1) \
        + rn * (alpha * er) * (alpha - 2.0 / r)
    km1 = np.maximum(k - 1, 0)
    km2 = np.maximum(k - 2, 0)
    xyz_km1 = _fast_power(xyz, km1)
    xyz_km2 = _fast_power(xyz, km2)
    kx, ky, kz = k[:, 0], k[:, 1], k[:, 2]
    dY = np.stack((kx * xyz_km1[..., 0] * xyz_k[..., 1] * xyz_k[..., 2],
                   ky * xyz_k[..., 0] * xyz_km1[..., 1] * xyz_k[..., 2],
                   kz * xyz_k[..., 0] * xyz_k[..., 1] * xyz_km1[..., 2]), axis=-1)
    d2Y = (kx * (kx - 1) * xyz_km2[..., 0] * xyz_k[..., 1] * xyz_k[..., 2]
           + ky * (ky - 1) * xyz_k[..., 0] * xyz_km2[..., 1] * xyz_k[..., 2]
           + kz * (kz - 1) * xyz_k[..., 0] * xyz_k[..., 1] * xyz_km2[..., 2])
    val = nc * R * Y
    grad = nc[:, None] * (nabla_R * Y[..., None] + R[..., None] * dY)
    lap = nc * (lap_R * Y + 2.0 * (nabla_R * dY).sum(-1) + R * d2Y)
    if derivative == 1 or derivative == [1]:
        return grad.sum(-1) if sum_grad else grad
    if derivative == 2 or derivative == [2]:
        return lap
    if list(derivative) == [0, 1, 2]:
        return val, grad, lap
    raise ValueError("derivative must be 0, 1, 2 or [0, 1, 2]")


def mo_values(ao, mo_scf, mo_modifier):
    """``MolecularOrbitals.forward`` (molecular_orbitals.py:79-95)."""
    return ao @ (np.asarray(mo_scf) * np.asarray(mo_modifier))


# ----------------------------------------------------------------------------
# electron-electron Pade Jastrow
# ----------------------------------------------------------------------------
def _tri_up(ne):
    row, col = [], []
    for i in range(ne - 1):
        for j in range(i + 1, ne):
            row.append(i)
            col.append(j)
    return np.array(row), np.array(col)


def pade_static_weight(nup, ndown):
    """``PadeJastrowKernel.get_static_weight`` (pade_jastrow_kernel.py:34-66):
    0.25 for same-spin pairs, 0.5 for opposite-spin pairs (upper triangle)."""
    ne = nup + ndown
    sw = np.full((ne, ne), 0.5)
    sw[:nup, :nup] = 0.25
    sw[nup:, nup:] = 0.25
    row, col = _tri_up(ne)
    return sw[row, col]


def jastrow_ee(pos, nup, ndown, w, derivative=0, sum_grad=True):
    """``JastrowFactorElectronElectron.forward`` and derivatives
    (jastrow_factor_electron_electron.py:124-260) with the Pade kernel
    (pade_jastrow_kernel.py:68-153) and the quadratic-form distance
    (electron_electron_distance.py:47-191, eps 41-45)."""
    pos = np.asarray(pos, dtype=np.float64)
    nb = pos.shape[0]
    ne = nup + ndown
    eps = 1e-16
    p = pos.reshape(nb, ne, 3)
    norm = (p ** 2).sum(-1)[..., None]
    dist = norm + np.swapaxes(norm, 1, 2) - 2.0 * (p @ np.swapaxes(p, 1, 2))
    eye = np.eye(ne)
    diag = np.einsum("bii->bi", dist)[:, :, None] * eye
    dist = np.sqrt(dist - diag + eps * eye)
    row, col = _tri_up(ne)
    r = dist[:, row, col]
    sw = pade_static_weight(nup, ndown)
    kern = sw * r / (1.0 + w * r)
    jast = np.exp(kern.sum(-1))[:, None]
    if derivative == 0:
        return jast
    # get_der_distance 128-149
    invr = 1.0 / (dist + eps * eye)
    pt = np.swapaxes(p, 1, 2)                   # (nb,3,ne)
    diff = pt[:, :, :, None] - pt[:, :, None, :]  # (nb,3,ne,ne)
    dr = (diff * invr[:, None])[:, :, row, col]   # (nb,3,npair)
    r_ = r[:, None, :]
    denom = 1.0 / (1.0 + w * r_)
    dker = sw * dr * denom - sw * w * r_ * dr * denom ** 2  # compute_derivative 84-117

    def first():
        out = np.zeros((nb, 3, ne))
        if sum_grad:
            dj = dker.sum(-2) * jast
            out = np.zeros((nb, ne))
            np.add.at(out, (slice(None), row), dj)
            np.add.at(out, (slice(None), col), -dj)
            return out
        dj = dker * jast[:, :, None]
        np.add.at(out, (slice(None), slice(None), row), dj)
        np.add.at(out, (slice(None), slice(None), col), -dj)
        return out

    def second():
        invr3 = 1.0 / (dist ** 3 + eps * eye)
        d2 = diff ** 2
        d2 = np.stack([d2[:, 1] + d2[:, 2], d2[:, 2] + d2[:, 0], d2[:, 0] + d2[:, 1]], axis=1)
        d2r = (d2 * invr3[:, None])[:, :, row, col]
        denom2 = denom ** 2
        drs = dr * dr
        d2k = (sw * d2r * denom - 2 * sw * w * drs * denom2 - sw * w * r_ * d2r * denom2
               + 2 * sw * w ** 2 * r_ * drs * denom ** 3).sum(-2)
        hess = np.zeros((nb, ne))
        np.add.at(hess, (slice(None), row), d2k)
        np.add.at(hess, (slice(None), col), d2k)
        part = np.zeros((nb, 3, ne))
        np.add.at(part, (slice(None), slice(None), row), dker)
        np.add.at(part, (slice(None), slice(None), col), -dker)
        return (hess + (part ** 2).sum(-2)) * jast

    if derivative == 1:
        return first()
    if derivative == 2:
        return second()
    if list(derivative) == [0, 1, 2]:
        return jast, first(), second()
    raise ValueError("bad derivative")


def jastrow_en(pos, atoms, w, derivative=0, sum_grad=True):
    """``JastrowFactorElectronNuclei.forward`` and derivatives
    (jastrow_factor_electron_nuclei.py:66-161) with the e-n Pade kernel
    (elec_nuclei/kernels/pade_jastrow_kernel.py:8-116, static weight 1) and the
    quadratic-form electron-nucleus distance (electron_nuclei_distance.py:60-190,
    eps 1e-16 in the derivative denominators)."""
    pos = np.asarray(pos, dtype=np.float64)
    atoms = np.asarray(atoms, dtype=np.float64).reshape(-1, 3)
    nb = pos.shape[0]
    p = pos.reshape(nb, -1, 3)
    eps = 1e-16
    norm = (p ** 2).sum(-1)[..., None]                     # (nb, ne, 1)
    norm_at = (atoms ** 2).sum(-1)[None, None, :]          # (1, 1, na)
    r = np.sqrt(norm + norm_at - 2.0 * p @ atoms.T)        # (nb, ne, na)
    kern = r / (1.0 + w * r)
    jast = np.exp(kern.sum((-1, -2)))[:, None]
    if derivative == 0:
        return jast
    diff = p[:, :, :, None] - atoms.T[None, None]          # (nb, ne, 3, na)
    dr = np.transpose(diff / (r[:, :, None, :] + eps), (0, 2, 1, 3))  # (nb, 3, ne, na)
    r_ = r[:, None]
    denom = 1.0 / (1.0 + w * r_)
    dker = dr * denom - w * r_ * dr * denom ** 2           # compute_derivative 48-82

    def first():
        if sum_grad:
            return dker.sum((1, 3)) * jast
        return dker.sum(3) * jast[:, :, None]

    def second():
        d2 = np.transpose(diff ** 2, (0, 2, 1, 3))         # (nb, 3, ne, na)
        d2 = np.stack([d2[:, 1] + d2[:, 2], d2[:, 2] + d2[:, 0], d2[:, 0] + d2[:, 1]], axis=1)
        d2r = d2 / (r[:, None] ** 3 + eps)
        drs = dr * dr
        d2k = (d2r * denom - 2 * w * drs * denom ** 2 - w * r_ * d2r * denom ** 2
               + 2 * w ** 2 * r_ * drs * denom ** 3)       # compute_second_derivative 84-116
        return (d2k.sum((1, 3)) + (dker.sum(3) ** 2).sum(1)) * jast

    if derivative == 1:
        return first()
    if derivative == 2:
        return second()
    if list(derivative) == [0, 1, 2]:
        return jast, first(), second()
    raise ValueError("bad derivative")


def combine_jastrow(terms, pos, derivative=0, sum_grad=True):
    """``CombineJastrow.forward`` (combine_jastrow.py:38-195): the product of
    the factors ``terms`` (callables with the (pos, derivative, sum_grad)
    signature above) with its product-rule derivatives."""
    def prod(v):
        out = v[0]
        for t in v[1:]:
            out = out * t
        return out

    def d1(vals, grads):
        if len(grads) == 1:
            return grads[0]
        return sum(prod(vals[:k] + [grads[k]] + vals[k + 1:]) for k in range(len(vals)))

    def d2(vals, grads, laps):
        if len(laps) == 1:
            return laps[0]
        out = sum(prod(vals[:k] + [laps[k]] + vals[k + 1:]) for k in range(len(vals)))
        wide = [v[..., None] for v in vals]
        for k in range(len(vals) - 1):
            for m in range(k + 1, len(vals)):
                t = list(wide)
                t[k], t[m] = grads[k], grads[m]
                out = out + 2.0 * prod(t).sum(1)
        return out

    vals = [f(pos, 0) for f in terms]
    if derivative == 0:
        return prod(vals)
    if derivative == 1:
        if sum_grad:
            return d1(vals, [f(pos, 1, True) for f in terms])
        return d1([v[..., None] for v in vals], [f(pos, 1, False) for f in terms])
    grads = [f(pos, 1, False) for f in terms]
    laps = [f(pos, 2) for f in terms]
    if derivative == 2:
        return d2(vals, grads, laps)
    return prod(vals), d1([v[..., None] for v in vals], grads), d2(vals, grads, laps)


# ----------------------------------------------------------------------------
# CI configurations and Slater pooling
# ----------------------------------------------------------------------------
def get_configs(configs, nup, ndown, nmo, spin=0):
    """``OrbitalConfigurations.get_configs`` (orbital_configurations.py:14-238)."""
    if isinstance(configs, tuple):
        return np.asarray(configs[0]), np.asarray(configs[1])
    c = configs.lower()
    gs_up, gs_dn = list(range(nup)), list(range(ndown))
    if c == "ground_state":
        return np.array([gs_up]), np.array([gs_dn])

    def orb_number(nel, norb):
        nocc = (nel // 2, nel // 2) if nel % 2 == 0 else (nel // 2 + 1, nel // 2)
        return nocc, (norb - nocc[0], norb - nocc[1])

    def singles(nocc, nvirt):
        cup, cdn = [gs_up], [gs_dn]
        for io in range(nup - 1, nup - 1 - nocc[0], -1):
            for iv in range(nup, nup + nvirt[0]):
                x = gs_up.copy()
                x[io] = iv
                cup.append(x)
                cdn.append(gs_dn)
        for io in range(ndown - 1, ndown - 1 - nocc[1], -1):
            for iv in range(ndown, ndown + nvirt[1]):
                x = gs_dn.copy()
                x[io] = iv
                cup.append(gs_up)
                cdn.append(x)
        return cup, cdn

    for prefix in ("cas(", "single_double(", "single("):
        if c.startswith(prefix):
            nel, norb = eval(c[len(prefix) - 1:])
            break
    else:
        raise ValueError("Config error")
    nocc, nvirt = orb_number(nel, norb)
    if c.startswith("single("):
        cup, cdn = singles(nocc, nvirt)
        return np.array(cup), np.array(cdn)
    if c.startswith("single_double("):
        cup, cdn = singles(nocc, nvirt)
        occ_up = list(range(nup - 1, nup - 1 - nocc[0], -1))
        vrt_up = list(range(nup, nup + nvirt[0]))
        occ_dn = list(range(ndown - 1, ndown - 1 - nocc[1], -1))
        vrt_dn = list(range(ndown, ndown + nvirt[1]))
        for ou in occ_up:
            for vu in vrt_up:
                for od in occ_dn:
                    for vd in vrt_dn:
                        xu = gs_up.copy()
                        xu[ou] = vu
                        xd = gs_dn.copy()
                        xd[od] = vd
                        cup.append(xu)
                        cdn.append(xd)
        from itertools import combinations
        for o1, o2 in combinations(occ_up, 2):
            for v1, v2 in combinations(vrt_up, 2):
                x = gs_up.copy()
                x[o1] = v2
                x[o2] = v1
                cup.append(x)
                cdn.append(gs_dn)
        for o1, o2 in combinations(occ_dn, 2):
            for v1, v2 in combinations(vrt_dn, 2):
                x = gs_dn.copy()
                x[o1] = v2
                x[o2] = v1
                cup.append(gs_up)
                cdn.append(x)
        return np.array(cup), np.array(cdn)
    # cas 180-214
    from itertools import combinations, product
    if spin != 0:
        raise ValueError("CAS active space not possible with spin polarized calculation")
    lo, hi = nup - nocc[0], nup + nvirt[0]
    frz = list(range(lo))
    cu = [frz + list(l) for l in combinations(range(lo, hi), nel // 2)]
    cd = [frz + list(l) for l in combinations(range(lo, hi), nel // 2)]
    conf = list(product(cu, cd))
    return np.array([x[0] for x in conf]), np.array([x[1] for x in conf])


class OraclePool:
    """``SlaterPooling`` (slater_pooling.py:11-849) with the index tables of
    ``get_unique_excitation`` (orbital_configurations.py:357-402) and
    ``ExcitationMask`` (orbital_projector.py:97-189), quirks included."""

    def __init__(self, config_method, configs, nup, ndown):
        self.method = config_method
        self.cup, self.cdn = np.asarray(configs[0]), np.asarray(configs[1])
        self.nup, self.ndown = nup, ndown
        self.max_up = int(self.cup.max()) + 1
        self.max_dn = int(self.cdn.max()) + 1
        self.explicit = config_method.startswith("cas(") or config_method == "explicit"
        # unique excitations, first-appearance order
        uu, ud, iu, idn = [], [], [], []
        for ic, (cu, cd) in enumerate(zip(self.cup, self.cdn)):
            su, sd = set(tuple(cu.tolist())), set(tuple(cd.tolist()))
            if ic == 0:
                gu, gd = su, sd
            eu = [list(gu.difference(su)), list(su.difference(gu))]
            ed = [list(gd.difference(sd)), list(sd.difference(gd))]
            if eu not in uu:
                uu.append(eu)
            if ed not in ud:
                ud.append(ed)
            iu.append(uu.index(eu))
            idn.append(ud.index(ed))
        self.index_unique_exc = (np.array(iu), np.array(idn))
        ncu, ncd = self.max_up - nup, self.max_dn - ndown
        self.single_up, self.single_dn, self.double_up, self.double_dn = [], [], [], []
        for eu, ed in zip(uu, ud):
            if len(eu[0]) == 1:
                self.single_up.append(eu[0][0] * ncu + eu[1][0] - nup)
            if len(ed[1]) == 1:
                self.single_dn.append(ed[0][0] * ncd + ed[1][0] - ndown)
        for eu, ed in zip(uu, ud):
            if len(eu[0]) == 2:
                for ie in eu[0]:
                    for io in eu[1]:
                        self.double_up.append(ie * ncu + io - nup)
            if len(ed[1]) == 2:
                for ie in eu[0]:        # orbital_projector.py:186 uses exc_up
                    for io in eu[1]:
                        self.double_dn.append(ie * ncd + io - ndown)
        # unique configs for det_explicit (orbital_projector.py:29-51)
        self.ucfg_up, self.iucfg_up = np.unique(self.cup, axis=0, return_inverse=True)
        self.ucfg_dn, self.iucfg_dn = np.unique(self.cdn, axis=0, return_inverse=True)
        self.iucfg_up = self.iucfg_up.reshape(-1)
        self.iucfg_dn = self.iucfg_dn.reshape(-1)

    # -- determinants ------------------------------------------------------
    def dets(self, mo):
        """``SlaterPooling.forward`` (64-80): det_explicit 96-111 or
        det_single_double 113-129 / det_unique_single_double 147-260."""
        nu, nd = self.nup, self.ndown
        nb = mo.shape[0]
        if self.explicit:
            du = np.stack([np.linalg.det(mo[:, :nu][:, :, c]) for c in self.ucfg_up], 0)
            dd = np.stack([np.linalg.det(mo[:, nu:][:, :, c]) for c in self.ucfg_dn], 0)
            return (du[self.iucfg_up] * dd[self.iucfg_dn]).T
        Aup, Adn = mo[:, :nu, :nu], mo[:, nu:, :nd]
        dAu, dAd = np.linalg.det(Aup), np.linalg.det(Adn)
        out_u, out_d = [dAu[:, None]], [dAd[:, None]]
        if self.method != "ground_state":
            mu = np.linalg.inv(Aup) @ mo[:, :nu, nu:self.max_up]
            md = np.linalg.inv(Adn) @ mo[:, nu:, nd:self.max_dn]
            mu, md = mu.reshape(nb, -1), md.reshape(nb, -1)
            if len(self.single_up):
                out_u.append(dAu[:, None] * mu[:, self.single_up])
                out_d.append(dAd[:, None] * md[:, self.single_dn])
            if len(self.double_up):
                t = mu[:, self.double_up].reshape(nb, -1, 2, 2)
                out_u.append(dAu[:, None] * (t[..., 0, 0] * t[..., 1, 1] - t[..., 0, 1] * t[..., 1, 0]))
                t = md[:, self.double_dn].reshape(nb, -1, 2, 2)
                out_d.append(dAd[:, None] * (t[..., 0, 0] * t[..., 1, 1] - t[..., 0, 1] * t[..., 1, 0]))
        du = np.concatenate(out_u, 1)
        dd = np.concatenate(out_d, 1)
        return du[:, self.index_unique_exc[0]] * dd[:, self.index_unique_exc[1]]

    # -- trace operator ----------------------------------------------------
    def operator(self, mo, bop):
        """``SlaterPooling.operator`` (262-306) with op=add:
        operator_ground_state 308-346, operator_explicit 348-409,
        operator_single_double 411-435 / operator_unique_single_double 437-636,
        op_single 639-673, op_multiexcitation 676-723."""
        nu, nd = self.nup, self.ndown
        nb = mo.shape[0]
        if self.explicit:
            ou = np.stack([np.trace(np.linalg.inv(mo[:, :nu][:, :, c]) @ bop[:, :nu][:, :, c],
                                    axis1=-2, axis2=-1) for c in self.ucfg_up], 0)
            od = np.stack([np.trace(np.linalg.inv(mo[:, nu:][:, :, c]) @ bop[:, nu:][:, :, c],
                                    axis1=-2, axis2=-1) for c in self.ucfg_dn], 0)
            return ou.T[:, self.iucfg_up] + od.T[:, self.iucfg_dn]
        iAu = np.linalg.inv(mo[:, :nu, :nu])
        iAd = np.linalg.inv(mo[:, nu:, :nd])
        ABu = iAu @ bop[:, :nu, :nu]
        ABd = iAd @ bop[:, nu:, :nd]
        gu = np.trace(ABu, axis1=-2, axis2=-1)[:, None]
        gd = np.trace(ABd, axis1=-2, axis2=-1)[:, None]
        if self.method == "ground_state":
            return gu + gd
        out_u, out_d = [gu], [gd]
        Avu = mo[:, :nu, nu:self.max_up]
        Avd = mo[:, nu:, nd:self.max_dn]
        mu = (iAu @ Avu).reshape(nb, -1)
        md = (iAd @ Avd).reshape(nb, -1)
        Mu = (iAu @ bop[:, :nu, nu:self.max_up] - iAu @ bop[:, :nu, :nu] @ iAu @ Avu).reshape(nb, -1)
        Md = (iAd @ bop[:, nu:, nd:self.max_dn] - iAd @ bop[:, nu:, :nd] @ iAd @ Avd).reshape(nb, -1)
        if len(self.single_up):
            out_u.append((1.0 / mu[:, self.single_up]) * Mu[:, self.single_up] + gu)
            out_d.append((1.0 / md[:, self.single_dn]) * Md[:, self.single_dn] + gd)
        if len(self.double_up):
            for (m, M, idx, g, out) in ((mu, Mu, self.double_up, gu, out_u),
                                        (md, Md, self.double_dn, gd, out_d)):
                T = np.linalg.inv(m[:, idx].reshape(nb, -1, 2, 2))
                mm = M[:, idx].reshape(nb, -1, 2, 2)
                out.append(np.trace(T @ mm, axis1=-2, axis2=-1) + g)
        ou = np.concatenate(out_u, 1)
        od = np.concatenate(out_d, 1)
        return ou[:, self.index_unique_exc[0]] + od[:, self.index_unique_exc[1]]


# ----------------------------------------------------------------------------
# the Slater-Jastrow wave function
# ----------------------------------------------------------------------------
class OracleSlaterJastrow:
    """``SlaterJastrow`` (slater_jastrow.py:30-482) + ``WaveFunction``
    (wf_base.py:49-247) in FP64 numpy."""

    def __init__(self, mol_like, configs="ground_state", include_all_mo=True,
                 jastrow_w=1.0, use_jastrow=True, fc_weight=None, mo_modifier=None,
                 bas_exp=None, jastrow_terms=None):
        """``jastrow_terms``: list of ("ee", w) / ("en", w) factors combined as
        CombineJastrow does; default [("ee", jastrow_w)] when use_jastrow."""
        b = mol_like.basis
        self.nup, self.ndown = int(mol_like.nup), int(mol_like.ndown)
        self.nelec = self.nup + self.ndown
        self.atom_coords = np.asarray(b.atom_coords_internal, dtype=np.float64)
        self.Z = np.asarray(mol_like.atomic_number, dtype=np.float64)
        self.basis = OracleBasis(b, self.atom_coords, bas_exp)
        self.configs_method = configs if isinstance(configs, str) else "explicit"
        self.configs = get_configs(configs, self.nup, self.ndown, int(b.nmo),
                                   getattr(mol_like, "spin", 0))
        self.nci = len(self.configs[0])
        self.highest_occ_mo = int(max(self.configs[0].max(), self.configs[1].max())) + 1
        mos = np.asarray(b.mos, dtype=np.float64)
        if not include_all_mo:
            mos = mos[:, : self.highest_occ_mo]
        self.mo_scf = mos
        self.mo_modifier = np.ones_like(mos) if mo_modifier is None else np.asarray(mo_modifier)
        self.pool = OraclePool(self.configs_method, self.configs, self.nup, self.ndown)
        if fc_weight is None:
            fc_weight = np.zeros(self.nci)
            fc_weight[0] = 1.0
        self.fc = np.asarray(fc_weight, dtype=np.float64).reshape(-1)
        self.use_jastrow = use_jastrow
        self.jastrow_w = float(jastrow_w)
        if jastrow_terms is None:
            jastrow_terms = [("ee", self.jastrow_w)] if use_jastrow else []
        self.jastrow_terms = [(k, float(w)) for k, w in jastrow_terms]
        self.use_jastrow = len(self.jastrow_terms) > 0
        self.en_atoms = np.asarray(mol_like.atom_coords, dtype=np.float64)

    @property
    def W(self):
        return self.mo_scf * self.mo_modifier

    def _factor(self, kind, w):
        if kind == "ee":
            return lambda pos, der=0, sg=True: jastrow_ee(pos, self.nup, self.ndown, w, der, sg)
        return lambda pos, der=0, sg=True: jastrow_en(pos, self.en_atoms, w, der, sg)

    def jastrow(self, pos, derivative=0, sum_grad=True):
        terms = [self._factor(k, w) for k, w in self.jastrow_terms]
        if len(terms) == 1:
            return terms[0](pos, derivative, sum_grad)
        return combine_jastrow(terms, pos, derivative, sum_grad)

    def forward(self, pos):
        """slater_jastrow.py:243-286 -> (nb, 1)."""
        ao = ao_values(self.basis, pos, 0)
        mo = ao @ self.W
        dets = self.pool.dets(mo)
        out = (dets @ self.fc)[:, None]
        if self.use_jastrow:
            out = self.jastrow(pos) * out
        return out

    def pdf(self, pos):
        """wf_base.py:241-247."""
        return (self.forward(pos) ** 2).reshape(-1)

    def kinetic_energy(self, pos):
        """kinetic_energy_jacobi (slater_jastrow.py:312-344) with
        get_kinetic_operator (449-482)."""
        ao, dao, d2ao = ao_values(self.basis, pos, [0, 1, 2])
        W = self.W
        mo = ao @ W
        bkin = d2ao @ W
        if self.use_jastrow:
            jast, djast, d2jast = self.jastrow(pos, [0, 1, 2], sum_grad=False)
            djast = np.swapaxes(djast, 1, 2) / jast[..., None]
            d2jast = d2jast / jast
            dmo = np.swapaxes(np.swapaxes(dao, 2, 3) @ W, 2, 3)
            bkin = bkin + 2 * (djast[:, :, None, :] * dmo).sum(-1) + d2jast[..., None] * mo
        bkin = -0.5 * bkin
        kin = self.pool.operator(mo, bkin)
        psi = self.pool.dets(mo)
        return ((kin * psi) @ self.fc / (psi @ self.fc))[:, None]

    def nuclear_potential(self, pos):
        """wf_base.py:72-95."""
        nb = pos.shape[0]
        p = np.zeros(nb)
        for ie in range(self.nelec):
            pe = pos[:, 3 * ie: 3 * ie + 3]
            for ia in range(len(self.Z)):
                r = np.sqrt(((pe - self.atom_coords[ia]) ** 2).sum(1))
                p += -self.Z[ia] / r
        return p[:, None]

    def electronic_potential(self, pos):
        """wf_base.py:49-70."""
        nb = pos.shape[0]
        p = np.zeros(nb)
        for i in range(self.nelec - 1):
            pi = pos[:, 3 * i: 3 * i + 3]
            for j in range(i + 1, self.nelec):
                r = np.sqrt(((pi - pos[:, 3 * j: 3 * j + 3]) ** 2).sum(1))
                p += 1.0 / r
        return p[:, None]

    def nuclear_repulsion(self):
        """wf_base.py:97-116."""
        v = 0.0
        for a in range(len(self.Z) - 1):
            for c in range(a + 1, len(self.Z)):
                r = np.sqrt(((self.atom_coords[a] - self.atom_coords[c]) ** 2).sum())
                v += self.Z[a] * self.Z[c] / r
        return v

    def local_energy(self, pos):
        """wf_base.py:184-215."""
        pos = np.asarray(pos, dtype=np.float64)
        return (self.kinetic_energy(pos) + self.nuclear_potential(pos)
                + self.electronic_potential(pos) + self.nuclear_repulsion())


# ----------------------------------------------------------------------------
# Metropolis sampling
# ----------------------------------------------------------------------------
def metropolis_sigma(step_size):
    """Per-coordinate standard deviation of the Gaussian proposal. The
    reference builds ``MultivariateNormal(0, sigma * I)`` with
    sigma = step / (2 sqrt(2 ln 2)) (metropolis.py:206-212), i.e. a variance
    of sigma, hence a standard deviation of sqrt(sigma)."""
    return float(np.sqrt(step_size / (2.0 * np.sqrt(2.0 * np.log(2.0)))))


def metropolis_replay(pdf, pos0, proposals, uniforms, ntherm=-1, ndecor=1,
                      nelec=None, move_type="all-elec", electron_index=None, trace=None):
    """``Metropolis.__call__`` (metropolis.py:85-177) with the random numbers
    supplied by the caller: ``proposals[istep, (iel), w, :]`` are the
    displacements (all-elec: (nstep, nw, 3*ne); single-electron moves:
    (nstep, nmove, nw, 3)) and ``uniforms[istep, (imove), w]`` the accept
    draws. Returns (snapshots (nsnap*nw, 3ne), accepted count, accept mask
    history). With a list ``trace``, each move appends (positions before the
    move, min(1, ratio) of the move) for decision-level comparisons."""
    eps = 1e-16
    pos = np.array(pos0, dtype=np.float64, copy=True)
    nw = pos.shape[0]
    nstep = proposals.shape[0]
    if ntherm >= nstep:
        raise ValueError("Thermalisation longer than trajectory")
    if ntherm < 0:
        ntherm = nstep + ntherm
    fx = pdf(pos)
    fx[fx == 0] = eps
    snaps, acc_hist, nacc, idecor = [], [], 0, 0
    for istep in range(nstep):
        if move_type == "all-elec":
            moves = [(None, proposals[istep], uniforms[istep])]
        else:
            moves = []
            nm = proposals.shape[1]
            for im in range(nm):
                iel = (electron_index[istep, im] if electron_index is not None
                       else np.full(nw, im))
                moves.append((iel, proposals[istep, im], uniforms[istep, im]))
        for iel, prop, u in moves:
            if iel is None:
                xn = pos + prop
            else:
                xn = pos.copy().reshape(nw, -1, 3)
                xn[np.arange(nw), iel, :] += prop
                xn = xn.reshape(nw, -1)
            fxn = pdf(xn)
            fxn[fxn == 0.0] = eps
            df = fxn / fx
            df[df > 1] = 1.0
            if trace is not None:
                trace.append((pos.copy(), df.copy()))
            idx = (df - u) >= 0
            pos[idx] = xn[idx]
            fx[idx] = fxn[idx]
            fx[fx == 0] = eps
            nacc += int(idx.sum())
            acc_hist.append(idx.copy())
        if istep >= ntherm:
            if idecor % ndecor == 0:
                snaps.append(pos.copy())
            idecor += 1
    return np.concatenate(snaps, 0), nacc, np.array(acc_hist)


def sampling_stats(eloc):
    """mean / var / error as ``SolverBase.single_point`` reports them
    (solver_base.py:371, wf_base.py:225-229); torch.var is unbiased."""
    e = np.asarray(eloc).reshape(-1)
    var = e.var(ddof=1)
    return e.mean(), var, np.sqrt(var / e.size)
