"""Write the synthetic aerosol model used by the .mie tests:
tests/golden/mie/synth_hg.mie and synth_peaked.mie, in the OPAC layout the reference reader
expects (code/OCRT_C/src/shared/mie_io.c:174-327): the angle count, a free
header, one spectral row per wavelength (wavelength in um, normalised
extinction, normalised scattering, single-scattering albedo, asymmetry,
extinction and scattering cross sections), then the three phase blocks P11,
P12, P33, each introduced by a TETA line naming the phase wavelengths, with
one row per angle from 180 to 0 degrees.

synth_hg.mie follows the synthetic aerosol of the batched-forward workload:
a Henyey-Greenstein P11 whose asymmetry falls with wavelength (0.72 at
400 nm, 0.64 at 1020 nm), a linear polarisation of the Rayleigh form scaled by
0.3 (P12 = -0.3 P11 sin^2 / (1 + cos^2)), and P33 blended the same way
(P33 = P11 (0.7 + 0.3 * 2 cos / (1 + cos^2))).  synth_peaked.mie has the same
polarisation on a forward-peaked P11 (35% in a g = 0.97 lobe), which the
log10-linear truncation acts on.  The angle grid is 0.1 degree
to 10 degrees and 0.5 degree beyond, so the tables are not uniform.  The
values are generated here; no external table is copied.

    python tests/golden/make_synthetic_mie.py
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "mie", "synth_hg.mie")

SPEC_WL = np.array([0.400, 0.443, 0.490, 0.555, 0.670, 0.765, 0.865, 1.020])
PHASE_WL = np.array([0.400, 0.550, 0.700, 0.865, 1.020])
PHASE_G = np.array([0.72, 0.70, 0.685, 0.66, 0.64])


def angles():
    a = np.concatenate([np.round(np.arange(0.0, 10.0 + 1e-9, 0.1), 3), np.arange(10.5, 180.0 + 1e-9, 0.5)])
    return a[::-1]                      # OPAC order: 180 -> 0


def hg(mu, g):
    return (1.0 - g * g) / (1.0 + g * g - 2.0 * g * mu) ** 1.5


def elements(theta_deg, g, peaked=False):
    mu = np.cos(np.radians(theta_deg))
    if peaked:
        # coarse-mode-like: a narrow forward lobe carrying 35% of the
        # scattering on top of a broad one (the log10-linear truncation
        # removes part of the lobe)
        p11 = 0.35 * hg(mu, 0.97) + 0.65 * hg(mu, g - 0.05)
    else:
        p11 = hg(mu, g)
    p12 = -0.3 * p11 * (1.0 - mu * mu) / (1.0 + mu * mu)
    p33 = p11 * (0.7 + 0.3 * 2.0 * mu / (1.0 + mu * mu))
    return p11, p12, p33


def write(path=OUT, peaked=False):
    th = angles()
    ang_ratio = (SPEC_WL / 0.555) ** -1.2
    ext = 0.8e-3 * ang_ratio              # cross sections of a nominal particle population
    ssa = np.interp(SPEC_WL, [0.4, 1.02], [0.97, 0.92])
    gs = np.interp(SPEC_WL, PHASE_WL, PHASE_G)
    lines = [f" {len(th)}",
             " synthetic aerosol model: Henyey-Greenstein P11, scaled Rayleigh-form polarisation",
             " wavelength  Nor_Ext_Co  Nor_Sca_Co  Sg_Sca_Alb  Asym_Par  Extinct_Co  Scatter_Co"]
    for w, e, s, g in zip(SPEC_WL, ext, ssa, gs):
        en = e / ext[3]
        lines.append(f" {w:.4f} {en:.6e} {en * s:.6e} {s:.6f} {g:.6f} {e:.6e} {e * s:.6e}")
    blocks = [elements(th[:, None], PHASE_G[None, :], peaked)[k] for k in range(3)]
    for name, b in zip(("P11", "P12", "P33"), blocks):
        lines.append(f" Phase Function ({name})")
        lines.append(" TETA " + " ".join(f"{w:.4f}" for w in PHASE_WL))
        for i, t in enumerate(th):
            lines.append(f" {t:8.3f} " + " ".join(f"{v:.8e}" for v in b[i]))
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


if __name__ == "__main__":
    print(write())
    print(write(os.path.join(HERE, "mie", "synth_peaked.mie"), peaked=True))
