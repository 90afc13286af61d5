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


BANDS_8 = np.array([412.0, 443.0, 490.0, 510.0, 555.0, 670.0, 765.0, 865.0])


def pure_water_b_synthetic(wl_nm):
    """Synthetic pure-water scattering b_w ~ 0.0019 (550/lambda)^4.32 per metre
    (the shape of the published seawater scattering curve, not its table)."""
    return 0.0019 * (550.0 / np.asarray(wl_nm, dtype=np.float64)) ** 4.32


def coupled_ocean_pixels(n_geom, seed=20261203 + 5):
    """Config 5 distribution: n_geom geometries x the 8 bands; per pixel-band
    a U[0.02, 0.5] and total b U[0.01, 1.0] per metre (pure water b_w plus a
    hydrosol carrying the rest), wind U[1, 12] m/s."""
    rng = np.random.default_rng(seed)
    sza, vza, raa = rng.uniform(0.0, 70.0, n_geom), rng.uniform(0.0, 60.0, n_geom), rng.uniform(0.0, 180.0, n_geom)
    wind = rng.uniform(1.0, 12.0, n_geom)
    rows = []
    for i in range(n_geom):
        for wl in BANDS_8:
            a = rng.uniform(0.02, 0.5)
            b = rng.uniform(0.01, 1.0)
            bw = float(pure_water_b_synthetic(wl))
            rows.append({"sza": sza[i], "vza": vza[i], "raa": raa[i], "wind": wind[i], "wavelength": float(wl),
                         "tau_r": float(tau_rayleigh_powerlaw(wl)), "a": a, "b_water": min(bw, b),
                         "b_particle": max(0.0, b - bw)})
    return rows
