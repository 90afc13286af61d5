"""The oracle's coupled atmosphere-ocean solve is pinned to the reference:
every case of tests/golden/reference_ocean.json (recipes R26 and R28 and
variations of geometry, wind, wavelength, absorption, node count and mode
count) must be reproduced from the water optical properties the reference
printed for it.

Tolerances follow the printed precision: TOA reflectances and transmittances
are printed with 11 significant digits (checked to 1e-9 relative), the
water-leaving radiances, irradiances and reflectances with 7 (checked to
1e-6), the diffuse attenuation coefficients to 1e-6 absolute."""
import pytest

from _helpers import load_golden_ocean, ocean_inputs_from_spec, ocean_ref_value, oracle_ocean, REF_OCEAN_KEYS

DOC = load_golden_ocean()


@pytest.mark.parametrize("spec", DOC["cases"], ids=[c["name"] for c in DOC["cases"]])
def test_oracle_matches_reference_ocean(oracle, spec):
    c, o, oc = ocean_inputs_from_spec(spec)
    got = oracle_ocean(oracle, c, o, oc)
    ref = spec["reference"]
    for ref_key, (got_key, tol) in REF_OCEAN_KEYS.items():
        r, g = ocean_ref_value(spec, ref_key), got[got_key]
        slack = 1e-6 if ref_key in ("Kd0minus", "Ku0minus") else 1e-15
        assert abs(g - r) <= tol * abs(r) + slack, (ref_key, g, r)
    assert got["orders_water"] == ref["orders"]


def test_oracle_published_ocean_recipes(oracle):
    for name, pub in DOC["published"].items():
        spec = next(s for s in DOC["cases"] if s["name"] == name)
        got = oracle_ocean(oracle, *ocean_inputs_from_spec(spec))
        assert abs(got["rho_I"] - pub["TOA_rho_I"]) <= 6e-11 * 10 * abs(pub["TOA_rho_I"])
        assert abs(got["Rrs_0plus_I"] - pub["Rrs0plus_I"]) <= 1e-6 * abs(pub["Rrs0plus_I"])
        assert abs(got["rrs_0minus_I"] - pub["rrs0minus_I"]) <= 1e-6 * abs(pub["rrs0minus_I"])
