"""Dispersive material models of the reference's ElectroMagnetic
(ElectroMagnetic.cpp:56-241), evaluated per wavelength on the host (a handful
of scalars per sphere) and handed to the library as relative parameters.

* ``gold(lambda, a, b, d)``: the hydrodynamic model ("GoldModel"): relative
  permittivity at omega and 2 omega from a five-term rational fit in
  (-i omega), and the surface / bulk chi(2) coefficients from the a, b, d
  parameters of the XML (ElectroMagnetic.cpp:72-157).
* ``silicon(lambda)``: "SiliconModel": n and k interpolated linearly on a
  10 nm grid from 0.25 um (ElectroMagnetic.cpp:160-224), constant chi(2).

The fit constants and the tabulated n, k are data that must equal the
reference's for parity; they are listed here as the reference lists them.
"""
from __future__ import annotations

import math

import numpy as np

C_LIGHT = 299792458.0          # consC (constants.cpp)
M_ELECTRON = 9.10938356e-31    # as ElectroMagnetic.cpp:138
Q_ELECTRON = 1.602176e-19      # as ElectroMagnetic.cpp:140

# rational-fit terms: eps_r = 1 + sum_i (a0 + s a1) / (b0 + s b1 + s^2 b2), s = -i omega
GOLD_A0 = np.array([2.00000339988256, 1.78238803442251e+32, 9.57114081841145e+26,
                    3.14102529060032e+24, 5.05628292785951e+31])
GOLD_A1 = np.array([0.0, 0.0, 8034165109695690.0, 106002790252082.0, 2.17631756605364e+16])
GOLD_B0 = np.array([1.0, 0.0, 1.39856631120507e+26, 5.98458120674188e+23, 1.70751028741696e+31])
GOLD_B1 = np.array([1.32629119239982e-15, 112272736197537.0, 7280057361739550.0,
                    4393809682455200.0, 3256258123271410.0])
GOLD_B2 = np.array([0.0, 1.0, 1.0, 1.0, 1.0])

# silicon n, k at 0.25 + 0.01 i micrometres, i = 0..120
N_SI = np.array([
    1.637, 1.737, 2.03, 2.84, 4.185, 5.049, 5.091, 5.085,
    5.135, 5.245, 5.423, 5.914, 6.82, 6.587, 6.025, 5.623,
    5.341, 5.11, 4.932, 4.79, 4.673, 4.572, 4.485, 4.412,
    4.349, 4.289, 4.235, 4.187, 4.145, 4.103, 4.073, 4.038,
    4.006, 3.977, 3.954, 3.931, 3.908, 3.888, 3.869, 3.851,
    3.835, 3.817, 3.805, 3.791, 3.776, 3.765, 3.753, 3.741,
    3.73, 3.719, 3.712, 3.701, 3.693, 3.684, 3.677, 3.669,
    3.662, 3.655, 3.646, 3.641, 3.636, 3.628, 3.622, 3.617,
    3.613, 3.61, 3.604, 3.598, 3.597, 3.59, 3.584, 3.584,
    3.578, 3.582, 3.579, 3.575, 3.572, 3.568, 3.565, 3.562,
    3.559, 3.556, 3.553, 3.549, 3.547, 3.545, 3.542, 3.54,
    3.537, 3.534, 3.533, 3.53, 3.527, 3.526, 3.524, 3.522,
    3.52, 3.518, 3.517, 3.515, 3.513, 3.512, 3.509, 3.509,
    3.506, 3.505, 3.503, 3.502, 3.501, 3.5, 3.499, 3.497,
    3.496, 3.496, 3.496, 3.493, 3.492, 3.492, 3.49, 3.488,
    3.487,
])

K_SI = np.array([
    3.5889, 3.9932, 4.5958, 5.1961, 5.3124, 4.29,
    3.6239, 3.2824, 3.0935, 2.9573, 2.9078, 2.9135,
    2.1403, 0.984, 0.5031, 0.3263, 0.2413, 0.1769,
    0.1377, 0.112, 0.0954, 0.0791, 0.0702, 0.0598,
    0.0538, 0.0485, 0.0438, 0.0395, 0.0348, 0.0299,
    0.028, 0.0266, 0.0237, 0.0219, 0.0201, 0.0185,
    0.0173, 0.0168, 0.0163, 0.0147, 0.0144, 0.0136,
    0.0128, 0.012, 0.0113, 0.0106, 0.01, 0.0093,
    0.0087, 0.0082, 0.0076, 0.0071, 0.0066, 0.0061,
    0.0057, 0.0053, 0.0049, 0.0045, 0.0041, 0.0038,
    0.0035, 0.0032, 0.0029, 0.0026, 0.0023, 0.0021,
    0.0019, 0.0017, 0.0015, 0.0013, 0.0011, 0.00098243,
    0.0008406, 0.00071334, 0.00059638, 0.0004902, 0.00039616, 0.00031437,
    0.00024048, 0.00017959, 0.00013043, 9.245e-05, 6.782e-05, 5.2168e-05,
    3.977e-05, 3.0217e-05, 2.2913e-05, 1.7068e-05, 1.2382e-05, 8.621e-06,
    5.6876e-06, 3.4275e-06, 1.7653e-06, 5.5561e-07, 2.3153e-07, 1.3904e-07,
    8.0863e-08, 4.794e-08, 2.7132e-08, 1.4318e-08, 5.8798e-09, 2.3352e-09,
    1.2714e-09, 7.5284e-10, 4.4799e-10, 2.7228e-10, 1.5856e-10, 8.7196e-11,
    4.2039e-11, 1.8128e-11, 1.0428e-11, 6.2911e-12, 3.903e-12, 2.6367e-12,
    1.7377e-12, 1.0428e-12, 6.0422e-13, 4.2895e-13, 2.0381e-13, 1.3785e-13,
    1.0901e-13,
])

SI_CHI = (65e-19, 3.5e-19, 1.3e-19)  # ksippp, ksiparppar, gamma


def _gold_eps(omega: float) -> complex:
    s = complex(0.0, -1.0) * omega
    total = 0j
    for i in range(5):
        total += (GOLD_A0[i] + s * GOLD_A1[i]) / (GOLD_B0[i] + s * GOLD_B1[i] + (s ** 2) * GOLD_B2[i])
    return 1.0 + total


def gold(wavelength: float, a: complex, b: complex, d: complex):
    """(eps_r, eps_r_SH, ksippp, ksiparppar, gamma) of the hydrodynamic model."""
    freq = C_LIGHT / wavelength
    omega = 2.0 * math.pi * freq
    eps = _gold_eps(omega)
    eps_sh = _gold_eps(2.0 * omega)
    scale = (eps - 1.0) * Q_ELECTRON / (M_ELECTRON * (2.0 * math.pi * freq) ** 2)
    return eps, eps_sh, -(a / 4.0) * scale, -(b / 2.0) * scale, -(d / 8.0) * scale


def _si_nk(lam_um: float):
    for i in range(len(K_SI)):
        lo, hi = 0.25 + i * 0.01, 0.25 + (i + 1) * 0.01
        if lo <= lam_um <= hi:
            break
    else:
        raise ValueError(f"SiliconModel covers 0.25-1.45 um (fundamental and second harmonic); "
                         f"got {lam_um} um")
    if i + 1 >= len(K_SI):
        raise ValueError(f"SiliconModel table ends at {0.25 + (len(K_SI) - 1) * 0.01:.2f} um")
    t = lam_um - lo
    n = N_SI[i] + (N_SI[i + 1] - N_SI[i]) / (hi - lo) * t
    k = K_SI[i] + (K_SI[i + 1] - K_SI[i]) / (hi - lo) * t
    return n, k


def silicon(wavelength: float):
    """(eps_r, eps_r_SH, ksippp, ksiparppar, gamma) of the silicon model."""
    lam_um = wavelength * 1e6
    nf, kf = _si_nk(lam_um)
    ns, ks = _si_nk(lam_um / 2.0)
    eps = complex(nf ** 2 - kf ** 2, 2.0 * nf * kf)
    eps_sh = complex(ns ** 2 - ks ** 2, 2.0 * ns * ks)
    return (eps, eps_sh) + SI_CHI
