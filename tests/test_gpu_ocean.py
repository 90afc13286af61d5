"""Coupled atmosphere-ocean solve on the GPU (ocrt_gb_solve_batch_ocean).

Every case of tests/golden/reference_ocean.json (recipes R26 and R28 of the
reference manual and variations of geometry, wind, wavelength, absorption,
node and mode count) is solved from the water optical properties the
reference printed and checked against the reference's own outputs:
  TOA reflectance: 1e-5 relative in I, 1e-4 absolute in Q and U (the bar);
  water-leaving reflectance Rrs(0+), rrs(0-) and the in-water irradiances:
  1e-4 relative (FP32 fields and interface operators against the FP64
  reference; the water-leaving signal is a few percent of the TOA signal).
The hydrosol and aerosol cases have no reference input path (hydrosol phase
moments only come from .mie tables there) and are checked against the FP64
oracle, whose coupled solve is pinned to the reference (test_oracle_ocean.py).
"""
import numpy as np
import pytest

from _helpers import (assert_parity, load_golden_ocean, ocean_inputs_from_spec, ocean_ref_value, oracle_ocean)

pytestmark = pytest.mark.gpu
DOC = load_golden_ocean()
WATER_REL = 1e-4


def _water_checks(got, ref_of, where):
    for gk, rk in (("Rrs_0plus_I", "Rrs0plus_I"), ("rrs_0minus_I", "rrs0minus_I"), ("Ed_0plus", "Ed0plus"),
                   ("Ed_0minus", "Ed0minus"), ("Lu_0plus_I", "Lu0plus"), ("Lu_0minus_I", "Lu0minus")):
        r = ref_of(rk)
        rel = abs(got[gk] - r) / abs(r)
        assert rel <= WATER_REL, f"{where}: {gk} {got[gk]:.7e} vs {r:.7e} (rel {rel:.1e})"
    for gk, rk in (("Rrs_0plus_Q", "Rrs0plus_Q"), ("Rrs_0plus_U", "Rrs0plus_U")):
        r = ref_of(rk)
        assert abs(got[gk] - r) <= WATER_REL * abs(ref_of("Rrs0plus_I")), (where, gk, got[gk], r)


@pytest.mark.parametrize("spec", DOC["cases"], ids=[c["name"] for c in DOC["cases"]])
def test_gpu_ocean_matches_reference(gpu, spec):
    c, o, oc = ocean_inputs_from_spec(spec)
    got = gpu.solve_ocean(c, o, oc)
    ref = spec["reference"]
    relI, dQ, dU = assert_parity(got, {"rho_I": ref["TOA_rho_I"], "rho_Q": ref["TOA_rho_Q"], "rho_U": ref["TOA_rho_U"]},
                                 spec["name"])
    _water_checks(got, lambda k: ocean_ref_value(spec, k), spec["name"])
    dw = abs(got["rho_water_I"] - ref["TOA_rho_water_direct_I"]) / abs(ref["TOA_rho_water_direct_I"])
    print(f"{spec['name']}: TOA rho_I rel {relI:.1e} |dQ| {dQ:.1e} |dU| {dU:.1e}; water-leaving at TOA rel {dw:.1e}; "
          f"Rrs(0+) rel {abs(got['Rrs_0plus_I'] - ref['Rrs0plus_I']) / ref['Rrs0plus_I']:.1e}")
    assert abs(got["Kd_0minus"] - ref["Kd0minus"]) <= 1e-3 * abs(ref["Kd0minus"]) + 2e-6
    assert got["orders_water"] in (ref["orders"], ref["orders"] + 1, ref["orders"] - 1)


def _hydrosol_case(A, g=0.92, L=80, wind=6.0, sza=35.0, vza=25.0, raa=60.0, wl=490.0, aer=None, **kw):
    from synthetic import hg_aerosol_moments
    c = A.default_case(surface="ocean", sza_deg=sza, vza_deg=vza, raa_deg=raa, wavelength_nm=wl, wind_speed=wind)
    o = A.default_opts(fourier_m_max=4, n_layers=30)
    args = dict(n_mu_water=16, m_max_water=4, depth_m=50.0, n_layers_water=60, max_orders_water=200)
    args.update(kw)
    oc = A.OceanHolder(0.08, 0.003, 0.2, hg_aerosol_moments(g, L), **args)
    return c, o, oc


def test_gpu_ocean_hydrosol_and_aerosol_vs_oracle(gpu, oracle):
    """Forward-peaked hydrosol (HG g = 0.92) in a 50 m column over an aerosol
    atmosphere: the configuration-5 medium at a test-sized node count."""
    from ocrt_gb300 import _abi as A
    from synthetic import hg_aerosol_moments
    aer = A.AerosolHolder(0.12, 0.95, *hg_aerosol_moments(0.7, 40))
    c, o, oc = _hydrosol_case(A)
    got = gpu.solve_ocean(c, o, oc, aer)
    ref = oracle_ocean(oracle, c, o, oc, aer)
    relI, dQ, dU = assert_parity(got, ref, "hydrosol + aerosol")
    _water_checks(got, lambda k: {"Rrs0plus_I": ref["Rrs_0plus_I"], "rrs0minus_I": ref["rrs_0minus_I"],
                                  "Ed0plus": ref["Ed_0plus"], "Ed0minus": ref["Ed_0minus"],
                                  "Lu0plus": ref["Lu_0plus_I"], "Lu0minus": ref["Lu_0minus_I"],
                                  "Rrs0plus_Q": ref["Rrs_0plus_Q"], "Rrs0plus_U": ref["Rrs_0plus_U"]}[k],
                  "hydrosol + aerosol")
    print(f"hydrosol + aerosol: TOA rho_I rel {relI:.1e}, Rrs rel "
          f"{abs(got['Rrs_0plus_I'] - ref['Rrs_0plus_I']) / ref['Rrs_0plus_I']:.1e}")


def test_gpu_ocean_batch_equals_single(gpu):
    """A mixed batch (per-pixel geometry, wind, water) gives each pixel's single solve."""
    from ocrt_gb300 import _abi as A
    specs = DOC["cases"][:3]
    ins = [ocean_inputs_from_spec(s, n_mu_water=16) for s in specs]
    res = gpu.solve_batch_ocean([i[0] for i in ins], [i[1] for i in ins], [i[2] for i in ins])
    for (c, o, oc), r in zip(ins, res):
        one = gpu.solve_ocean(c, o, oc)
        for k in ("rho_I", "rho_Q", "rho_U", "Rrs_0plus_I", "Ed_0minus", "Lu_0minus_I"):
            assert abs(r[k] - one[k]) <= 1e-12 * max(1.0, abs(one[k])), k


def test_gpu_ocean_rejects_unsupported(gpu):
    from ocrt_gb300 import _abi as A
    c, o, oc = _hydrosol_case(A)
    c.wind_speed = 0.0
    with pytest.raises(gpu.OcrtError) as e:
        gpu.solve_ocean(c, o, oc)
    assert e.value.rc == A.OCRT_ERR_UNSUPPORTED
    c, o, oc = _hydrosol_case(A)
    o.pssa = 1
    with pytest.raises(gpu.OcrtError) as e:
        gpu.solve_ocean(c, o, oc)
    assert e.value.rc == A.OCRT_ERR_UNSUPPORTED
    c, o, oc = _hydrosol_case(A)
    c.surface = A.SURFACE_BLACK
    with pytest.raises(gpu.OcrtError) as e:
        gpu.solve_ocean(c, o, oc)
    assert e.value.rc == A.OCRT_ERR_ARGS
