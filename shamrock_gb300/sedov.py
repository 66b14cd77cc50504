"""Sedov-Taylor point-blast solution, the validation aid of the Sedov set-ups.

Mirrors the reference's ``shamrock.phys.SedovTaylor`` (shamphys/SedovTaylor.hpp:34-50,
bound in shampylib/src/pyShamphys.cpp:371-380): ``SedovTaylor().get_value(r)`` returns
(rho, v_r, P) at radius r of a spherical blast of energy 1 in a cold uniform gas of
density 1, gamma = 5/3, at t = 0.1.  The reference interpolates a 3000-point table on
[1e-6, 0.5] (shamphys/src/SedovTaylor.cpp:67-83); here the solution is evaluated from
the closed-form similarity solution instead, for any gamma, energy, density and time.

Method: the standard-case (uniform ambient density) closed form of Sedov (1959) as
written by Kamm & Timmes, "On efficient generation of numerically robust Sedov
solutions" (LA-UR-07-2849, 2007).  With j = 3 and the similarity variable V between
v0 = 2/(5 gamma) (centre) and v2 = 4/(5 (gamma + 1)) (shock),
    x1 = a V,  x2 = b (c V - 1),  x3 = d (1 - e V),  x4 = b (1 - c V / gamma),
    lambda = r / R = x1^-a0 x2^-a2 x3^-a1,
    u / u_s = x1 lambda,  rho / rho_s = x2^a3 x3^a4 x4^a5,  P / P_s = x1^(3 a0) x3^(a4 - 2 a1) x4^(1 + a5),
with the shock values u_s = 2 R'/(gamma + 1), rho_s = rho0 (gamma + 1)/(gamma - 1),
P_s = 2 rho0 R'^2/(gamma + 1), R' = 2R/(5t).  The shock radius R = (E t^2/(alpha rho0))^(1/5)
follows from the energy integral
    E = 4 pi R^3 rho0 R'^2 2/(gamma^2 - 1) Int_0^1 (rho/rho_s (u/u_s)^2 + P/P_s) lambda^2 d lambda,
evaluated here by Gauss-Legendre quadrature in s = log x2 (x2 runs from 0 at the centre
to 1 at the shock; the parametrisation keeps the centre, where lambda ~ x2^(-a2) with a
small exponent, resolvable in double precision).
"""

from __future__ import annotations

import math

import numpy as np

__all__ = ["SedovTaylor"]


class SedovTaylor:
    """Spherical Sedov-Taylor blast (j = 3) in a uniform cold medium.

    Parameters default to the reference's tabulated case: gamma 5/3, blast energy 1,
    ambient density 1, time 0.1 (shock radius 0.45849)."""

    _S_MIN = -5000.0  # log x2 at the innermost bisection bracket (lambda ~ 1e-334)

    def __init__(self, gamma: float = 5.0 / 3.0, t: float = 0.1, e_blast: float = 1.0,
                 rho0: float = 1.0):
        if not (1.0 < gamma < 2.0):
            raise ValueError("SedovTaylor: the standard-case closed form needs 1 < gamma < 2")
        if not (t > 0 and e_blast > 0 and rho0 > 0):
            raise ValueError("SedovTaylor: t, e_blast and rho0 must be positive")
        g = float(gamma)
        j = 3.0
        self.gamma, self.t, self.e_blast, self.rho0 = g, float(t), float(e_blast), float(rho0)
        # exponents and coefficients of the standard case (w = 0)
        self._a = (j + 2) * (g + 1) / 4
        self._b = (g + 1) / (g - 1)
        self._c = (j + 2) * g / 2
        self._d = (j + 2) * (g + 1) / ((j + 2) * (g + 1) - 2 * (2 + j * (g - 1)))
        self._e = (2 + j * (g - 1)) / 2
        self._a0 = 2 / (j + 2)
        self._a2 = -(g - 1) / (2 * (g - 1) + j)
        self._a1 = (j + 2) * g / (2 + j * (g - 1)) * (2 * j * (2 - g) / (g * (j + 2) ** 2) - self._a2)
        self._a3 = j / (2 * (g - 1) + j)
        self._a4 = (j + 2) * j / (j * (2 - g)) * self._a1
        self._a5 = -2 * j / (j * (2 - g))
        self.v0 = 2 / ((j + 2) * g)
        self.v2 = 4 / ((j + 2) * (g + 1))
        self.alpha = self._energy_constant()
        self.shock_radius = (self.e_blast * self.t ** 2 / (self.alpha * self.rho0)) ** 0.2
        rdot = 0.4 * self.shock_radius / self.t
        self.shock_speed = rdot
        self.u_s = 2 * rdot / (g + 1)
        self.rho_s = self.rho0 * (g + 1) / (g - 1)
        self.p_s = 2 * self.rho0 * rdot * rdot / (g + 1)

    # ---- the similarity curve, parametrised by s = log x2 in (-inf, 0]
    def _logs(self, s):
        x2 = np.exp(s)
        V = (1.0 + x2 / self._b) / self._c
        lx1 = np.log(self._a * V)
        lx3 = np.log(self._d * (1.0 - self._e * V))
        lx4 = np.log(self._b * (1.0 - self._c * V / self.gamma))
        llam = -self._a0 * lx1 - self._a2 * s - self._a1 * lx3
        return V, x2, lx1, lx3, lx4, llam

    def _profile(self, s):
        """(lambda, u/u_s, rho/rho_s, P/P_s) along the curve."""
        V, x2, lx1, lx3, lx4, llam = self._logs(s)
        lam = np.exp(llam)
        f = np.exp(lx1) * lam
        gr = np.exp(self._a3 * s + self._a4 * lx3 + self._a5 * lx4)
        h = np.exp(3 * self._a0 * lx1 + (self._a4 - 2 * self._a1) * lx3 + (1 + self._a5) * lx4)
        return lam, f, gr, h

    def _dllam_ds(self, s):
        V, x2, *_ = self._logs(s)
        dV = x2 / (self._b * self._c)
        return -self._a0 * dV / V - self._a2 + self._a1 * self._e * dV / (1.0 - self._e * V)

    def _energy_constant(self):
        """alpha = E t^2 / (rho0 R^5)."""
        xg, wg = np.polynomial.legendre.leggauss(32)
        edges = np.concatenate([np.linspace(-80.0, -10.0, 15), np.linspace(-10.0, 0.0, 41)[1:]])
        total = 0.0
        for lo, hi in zip(edges[:-1], edges[1:]):
            s = 0.5 * (hi - lo) * xg + 0.5 * (hi + lo)
            lam, f, gr, h = self._profile(s)
            integrand = (gr * f * f + h) * lam ** 3 * self._dllam_ds(s)
            total += 0.5 * (hi - lo) * float(np.dot(wg, integrand))
        g = self.gamma
        return 4 * math.pi * 0.16 * 2 / (g * g - 1) * total

    def _s_of_lambda(self, lam):
        """Bisection for s with lambda(s) = lam, 0 < lam < 1 (lambda increases with s)."""
        target = np.log(lam)
        lo = np.full(lam.shape, self._S_MIN)
        hi = np.zeros(lam.shape)
        for _ in range(120):
            mid = 0.5 * (lo + hi)
            below = self._logs(mid)[5] < target
            lo = np.where(below, mid, lo)
            hi = np.where(below, hi, mid)
        return 0.5 * (lo + hi)

    def profile(self, r):
        """Vectorised (rho, v_r, P) at radii r (array-like, r >= 0)."""
        r = np.asarray(r, dtype=np.float64)
        if np.any(r < 0) or not np.all(np.isfinite(r)):
            raise ValueError("SedovTaylor: radii must be finite and >= 0")
        lam = r / self.shock_radius
        rho = np.full(r.shape, self.rho0)
        vr = np.zeros(r.shape)
        p = np.zeros(r.shape)
        inside = lam < 1.0
        centre = lam == 0.0
        mid = inside & ~centre
        if np.any(mid):
            s = self._s_of_lambda(lam[mid])
            _, f, gr, h = self._profile(s)
            rho[mid] = self.rho_s * gr
            vr[mid] = self.u_s * f
            p[mid] = self.p_s * h
        if np.any(centre):
            _, _, gr, h = self._profile(np.array([-np.inf]))
            rho[centre] = 0.0
            vr[centre] = 0.0
            p[centre] = self.p_s * h[0]
        return rho, vr, p

    def get_value(self, x: float):
        """(rho, v_r, P) at radius x, as the reference's SedovTaylor.get_value."""
        rho, vr, p = self.profile(np.array([abs(float(x))]))
        return float(rho[0]), float(vr[0]), float(p[0])
