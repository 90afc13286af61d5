"""Seeded synthetic inputs with the shapes of the benchmark configurations.

TEST INFRASTRUCTURE and workload generator: the aerosol expansion used by
every configuration is frozen here so the oracle, the fixtures, the tests and
bench.py all see the same inputs.

Synthetic aerosol (configs 2-4): beta_l = (2l+1) g^l (Henyey-Greenstein),
gamma_2 and alpha_2 equal to 0.3 x the molecular (Rayleigh-form) values of
rt_molecular_phase.c:12-18 at depolarisation 0.0279, every other gamma/alpha/
zeta moment zero.  This is the frozen reading of "polarisation terms scaled
from Rayleigh form by 0.3".
"""
import numpy as np

DEPOL = 0.0279


def rayleigh_form_moments():
    A = 2.0 * (1.0 - DEPOL) / (2.0 + DEPOL)
    return {"beta2": 0.5 * A, "gamma2": -A * np.sqrt(1.5), "alpha2": 3.0 * A}


def hg_aerosol_moments(g, L, pol_scale=0.3):
    l = np.arange(L + 1, dtype=np.float64)
    beta = (2.0 * l + 1.0) * g ** l
    gamma = np.zeros(L + 1)
    alpha = np.zeros(L + 1)
    zeta = np.zeros(L + 1)
    mol = rayleigh_form_moments()
    gamma[2] = pol_scale * mol["gamma2"]
    alpha[2] = pol_scale * mol["alpha2"]
    return beta, gamma, alpha, zeta


def tau_rayleigh_powerlaw(wl_nm, tau_555=0.0945, exponent=4.08):
    """Synthetic Rayleigh depth tau ~ lambda^-4.08 anchored at 0.0945 (555 nm)."""
    return tau_555 * (np.asarray(wl_nm, dtype=np.float64) / 555.0) ** (-exponent)


BANDS_10 = np.linspace(412.0, 865.0, 10)


def batched_forward_pixels(n=4096, seed=20261203 + 3):
    """Config 3 distribution: uneven geometry, layers, wavelength, AOD, wind, g, SSA."""
    rng = np.random.default_rng(seed)
    p = {
        "sza": rng.uniform(0.0, 80.0, n),
        "vza": rng.uniform(0.0, 70.0, n),
        "raa": rng.uniform(0.0, 180.0, n),
        "aod": np.exp(np.log(0.1) + 0.6 * rng.standard_normal(n)),
        "n_layers": rng.choice(np.array([50, 100, 200, 400]), n),
        "wavelength": rng.choice(BANDS_10, n),
        "wind": rng.uniform(1.0, 12.0, n),
        "g": rng.uniform(0.6, 0.8, n),
        "ssa": rng.uniform(0.85, 0.99, n),
    }
    p["tau_r"] = tau_rayleigh_powerlaw(p["wavelength"])
    return p
