"""The Sedov-Taylor similarity solution (shamrock_gb300.sedov) against the reference's
tabulated solution (src/shamphys/src/sedov_soluce_arrays.hpp, subsampled into
tests/golden/sedov_taylor_table.json by tests/golden/extract_golden.py) and against the
conservation laws the solution obeys."""

import json
import os

import numpy as np
import pytest

from shamrock_gb300.sedov import SedovTaylor

HERE = os.path.dirname(os.path.abspath(__file__))


def _table():
    with open(os.path.join(HERE, "golden", "sedov_taylor_table.json")) as f:
        return json.load(f)


def test_matches_reference_table():
    """rho and v_r agree with the reference's 7-digit table to 1e-5 everywhere but the
    two table points that straddle the shock; P agrees to 1e-5 outside r = 0.02.  Inside
    it the table's pressure wanders between 0.77212 and 0.77281 around the closed form's
    0.772384 (the table generator's noise near the centre, at most 5.6e-4 relative),
    so the tolerance there is 6e-4."""
    t = _table()
    c = t["case"]
    st = SedovTaylor(gamma=c["gamma"], t=c["t"], e_blast=c["e_blast"], rho0=c["rho0"])
    r = np.array(t["r_theo"])
    rho, vr, p = st.profile(r)
    # the table places the shock between its points 0.4584862 and 0.458653
    assert 0.4584862 < st.shock_radius < 0.458653
    away = np.abs(r - st.shock_radius) > 2e-4
    ref_rho, ref_v, ref_p = (np.array(t[k]) for k in ("rho_theo", "vr_theo", "p_theo"))
    assert np.all(np.abs(rho - ref_rho)[away] <= 1e-5 * np.maximum(ref_rho[away], 1e-3))
    assert np.all(np.abs(vr - ref_v)[away] <= 1e-5 * np.maximum(np.abs(ref_v[away]), 1e-2))
    outer = away & (r > 0.02)
    assert np.all(np.abs(p - ref_p)[outer] <= 1e-5 * np.maximum(ref_p[outer], 1e-3))
    inner = r <= 0.02
    assert np.all(np.abs(p - ref_p)[inner] <= 6e-4 * ref_p[inner])


def test_get_value_api():
    st = SedovTaylor()
    rho, vr, p = st.get_value(0.3)
    assert isinstance(rho, float) and isinstance(vr, float) and isinstance(p, float)
    # ambient state beyond the shock, as the reference's table ends (rho 1, v 0, P 0)
    assert st.get_value(0.6) == (1.0, 0.0, 0.0)
    # post-shock (Rankine-Hugoniot, strong shock) just inside R
    rho, vr, p = st.get_value(st.shock_radius * (1 - 1e-12))
    g = 5.0 / 3.0
    assert rho == pytest.approx((g + 1) / (g - 1), rel=1e-9)
    assert vr == pytest.approx(2 / (g + 1) * st.shock_speed, rel=1e-9)
    assert p == pytest.approx(2 / (g + 1) * st.shock_speed ** 2, rel=1e-9)


@pytest.mark.parametrize("gamma,alpha", [(1.4, 0.851072), (5.0 / 3.0, 0.493590)])
def test_energy_constant(gamma, alpha):
    """alpha = E t^2/(rho0 R^5) against the published values for the spherical blast
    (Kamm & Timmes 2007, their table of alpha: 0.851072 for gamma 1.4)."""
    assert SedovTaylor(gamma=gamma).alpha == pytest.approx(alpha, abs=2e-6)


@pytest.mark.parametrize("gamma", [1.4, 5.0 / 3.0])
def test_conservation(gamma):
    """The profile carries the blast energy and the swept-up mass."""
    st = SedovTaylor(gamma=gamma, t=0.05, e_blast=2.0, rho0=0.5)
    r = np.linspace(0.0, st.shock_radius * (1 - 1e-12), 100001)
    rho, vr, p = st.profile(r)
    shell = 4 * np.pi * r * r
    energy = np.trapezoid((0.5 * rho * vr * vr + p / (gamma - 1)) * shell, r)
    mass = np.trapezoid(rho * shell, r)
    assert energy == pytest.approx(2.0, rel=1e-6)
    assert mass == pytest.approx(0.5 * 4 / 3 * np.pi * st.shock_radius ** 3, rel=1e-6)
