"""Gaussian basis-set tables for the elements the VMC hot path is run on.

Each element maps to an ordered list of shells ``(l, exponents, coefficients)``
where ``coefficients`` has one column per general contraction (the layout of
an NWChem/BSE basis file, shells sorted by angular momentum as pyscf stores
them).

* ``sto-3g``: Hehre, Stewart, Pople, J. Chem. Phys. 51, 2657 (1969); the
  values are the standard published STO-3G exponents and contraction
  coefficients.
* ``cc-pvdz``: Dunning, J. Chem. Phys. 90, 1007 (1989) (H, C, O); the
  [9s4p1d/3s2p1d] and [4s1p/2s1p] contraction layout with the published
  exponents and coefficients. The coefficients are used as tabulated (pyscf
  renormalises them internally, which only rescales each contracted AO).
"""

STO3G_S_COEF = [0.15432897, 0.53532814, 0.44463454]
STO3G_SP_S_COEF = [-0.09996723, 0.39951283, 0.70011547]
STO3G_SP_P_COEF = [0.15591627, 0.60768372, 0.39195739]


def _col(c):
    return [[x] for x in c]


BASIS_TABLES = {
    "sto-3g": {
        "H": [(0, [3.42525091, 0.62391373, 0.16885540], _col(STO3G_S_COEF))],
        "He": [(0, [6.36242139, 1.15892300, 0.31364979], _col(STO3G_S_COEF))],
        "Li": [
            (0, [16.1195750, 2.9362007, 0.7946505], _col(STO3G_S_COEF)),
            (0, [0.6362897, 0.1478601, 0.0480887], _col(STO3G_SP_S_COEF)),
            (1, [0.6362897, 0.1478601, 0.0480887], _col(STO3G_SP_P_COEF)),
        ],
        "C": [
            (0, [71.6168370, 13.0450960, 3.5305122], _col(STO3G_S_COEF)),
            (0, [2.9412494, 0.6834831, 0.2222899], _col(STO3G_SP_S_COEF)),
            (1, [2.9412494, 0.6834831, 0.2222899], _col(STO3G_SP_P_COEF)),
        ],
        "N": [
            (0, [99.1061690, 18.0523120, 4.8856602], _col(STO3G_S_COEF)),
            (0, [3.7804559, 0.8784966, 0.2857144], _col(STO3G_SP_S_COEF)),
            (1, [3.7804559, 0.8784966, 0.2857144], _col(STO3G_SP_P_COEF)),
        ],
        "O": [
            (0, [130.7093200, 23.8088610, 6.4436083], _col(STO3G_S_COEF)),
            (0, [5.0331513, 1.1695961, 0.3803890], _col(STO3G_SP_S_COEF)),
            (1, [5.0331513, 1.1695961, 0.3803890], _col(STO3G_SP_P_COEF)),
        ],
    },
    "cc-pvdz": {
        "H": [
            (0, [13.01, 1.962, 0.4446, 0.122],
             _col([0.019685, 0.137977, 0.478148, 0.50124])),
            (0, [0.122], [[1.0]]),
            (1, [0.727], [[1.0]]),
        ],
        "C": [
            (0, [6665.0, 1000.0, 228.0, 64.71, 21.06, 7.495, 2.797, 0.5215, 0.1596],
             [[0.000692, -0.000146], [0.005329, -0.001154], [0.027077, -0.005725],
              [0.101718, -0.023312], [0.274740, -0.063955], [0.448564, -0.149981],
              [0.285074, -0.127262], [0.015204, 0.544529], [-0.003191, 0.580496]]),
            (0, [0.1596], [[1.0]]),
            (1, [9.439, 2.002, 0.5456, 0.1517],
             _col([0.038109, 0.209480, 0.508557, 0.468842])),
            (1, [0.1517], [[1.0]]),
            (2, [0.55], [[1.0]]),
        ],
        "O": [
            (0, [11720.0, 1759.0, 400.8, 113.7, 37.03, 13.27, 5.025, 1.013, 0.3023],
             [[0.000710, -0.000160], [0.005470, -0.001263], [0.027837, -0.006267],
              [0.104800, -0.025716], [0.283062, -0.070924], [0.448719, -0.165411],
              [0.270952, -0.116955], [0.015458, 0.557368], [-0.002585, 0.572759]]),
            (0, [0.3023], [[1.0]]),
            (1, [17.70, 3.854, 1.046, 0.2753],
             _col([0.043018, 0.228913, 0.508728, 0.460531])),
            (1, [0.2753], [[1.0]]),
            (2, [1.185], [[1.0]]),
        ],
    },
}

# Valence-state ionisation energies (eV) used by the extended-Hueckel MO guess:
# (core s, valence s, valence p, polarisation d).
HUCKEL_VSIE = {
    "H": (-13.6, -13.6, -4.0, -2.0),
    "He": (-24.6, -24.6, -4.0, -2.0),
    "Li": (-64.0, -5.4, -3.5, -2.0),
    "C": (-290.0, -21.4, -11.4, -2.0),
    "N": (-400.0, -26.0, -13.4, -2.0),
    "O": (-540.0, -32.3, -14.8, -2.0),
}

ATOMIC_NUMBER = {"H": 1, "He": 2, "Li": 3, "Be": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9}
