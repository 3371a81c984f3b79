"""Material tables of the reference, restated for callers without the Fortran host.

The Fortran driver builds these tables itself (InitPrtclProperty /
InitWallProperty, src/DEM/Prtcl_Property.f90:62-195) and uploads them through
sdem_set_types; this module builds the same numbers for Python callers, with
the reference's order of floating-point operations (Python floats are IEEE
doubles; ** and math.log/sqrt call the same libm as gfortran).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Sequence

import numpy as np

CFT_LSD = 1
CFT_NLIN = 2
PI = 3.141592653589793238462643383279502884
BP_SIZE = 11  # RadEff, MassEff, Kn, Kt, Cn, Ct, en, et, mu_s, mu_k, mu_roll


@dataclass
class PureProperty:
    """type PureProperty, Prtcl_Property.f90:14-26."""
    radius: float
    density: float
    youngs: float
    poisson: float
    mass: float
    volume: float
    inertia: float


def pure_property(diameter: float, density: float, youngs: float, poisson: float) -> PureProperty:
    """Prtcl_Property.f90:121-128: Volume = 4/3*Pi*R**3, Mass, Inertia = 2/5*Mass*R**2."""
    r = 0.5 * diameter
    vol = 4.0 / 3.0 * PI * (r * r * r)
    mass = density * vol
    inertia = 2.0 / 5.0 * mass * (r * r)
    return PureProperty(r, density, youngs, poisson, mass, vol, inertia)


def wall_pure_property(youngs: float, poisson: float) -> PureProperty:
    """Prtcl_Property.f90:176-185: walls are infinitely large and heavy (1e50)."""
    return PureProperty(1.0e50, 1.0e50, youngs, poisson, 1.0e50, 1.0e50, 1.0e50)


def binary_property(cf_type: int, pari: PureProperty, parj: PureProperty, mu_s: float, mu_k: float,
                    mu_roll: float, e_n: float, e_t: float, iswall: bool) -> np.ndarray:
    """clc_BnryPrtcl_Prop, Prtcl_Property.f90:200-247 -> 11 doubles."""
    out = np.zeros(BP_SIZE)
    if not iswall:
        rad_eff = (pari.radius * parj.radius) / (pari.radius + parj.radius)
        mass_eff = (pari.mass * parj.mass) / (pari.mass + parj.mass)
    else:
        rad_eff = pari.radius
        mass_eff = pari.mass
    pri, prj = pari.poisson, parj.poisson
    g_i = pari.youngs / (2.0 * (1.0 + pri))
    g_j = parj.youngs / (2.0 * (1.0 + prj))
    e_eff = 1.0 / ((1.0 - pri * pri) / pari.youngs + (1.0 - prj * prj) / parj.youngs)
    g_eff = 1.0 / ((2.0 - pri) / g_i + (2.0 - prj) / g_j)
    kappa = ((1.0 - pri) / g_i + (1.0 - prj) / g_j) / ((1.0 - 0.5 * pri) / g_i + (1.0 - 0.5 * prj) / g_j)
    kappa = abs(kappa)
    eta = math.log(e_n)
    eta = eta * eta
    kn = kt = cn = 0.0
    if cf_type == CFT_LSD:
        kn = 1.2024 * (math.sqrt(mass_eff) * (e_eff * e_eff) * rad_eff) ** 0.4
        kt = kappa * kn
        cn = -2.0 * math.log(e_n) * math.sqrt(mass_eff * kn) / math.sqrt(PI * PI + eta)
    elif cf_type == CFT_NLIN:
        k_hertz = 4.0 / 3.0 * e_eff * math.sqrt(rad_eff)
        kn = k_hertz
        kt = 16.0 / 3.0 * g_eff * math.sqrt(rad_eff)
        cn = -2.2664 * math.log(e_n) * math.sqrt(mass_eff * k_hertz) / math.sqrt(eta + 10.1354)
    out[:] = (rad_eff, mass_eff, kn, kt, cn, 0.0, e_n, e_t, mu_s, mu_k, mu_roll)
    return out


@dataclass
class Tables:
    """Everything sdem_set_types uploads."""
    radius: np.ndarray   # (nT,)
    mass: np.ndarray     # (nT,)
    inertia: np.ndarray  # (nT,)
    bpp: np.ndarray      # (nT*nT*11,), record (i,j) at j*nT+i
    bpw: np.ndarray      # (nT*nWT*11,), record (i,w) at w*nT+i

    @property
    def n_types(self) -> int:
        return len(self.radius)

    @property
    def n_wall_types(self) -> int:
        return len(self.bpw) // (BP_SIZE * self.n_types)


def build_tables(cf_type: int, diameters: Sequence[float], densities: Sequence[float],
                 youngs_p: Sequence[float], poisson_p: Sequence[float],
                 pp: tuple, youngs_w: Sequence[float], poisson_w: Sequence[float], pw: tuple,
                 quirk_same_type: bool = True) -> Tables:
    """InitPrtclProperty + InitWallProperty (Prtcl_Property.f90:120-143, 176-194).

    pp / pw = (mu_s, mu_k, mu_roll, e_n, e_t) of the particle-particle and
    particle-wall groups.  quirk_same_type reproduces Prtcl_Property.f90:137-138,
    where both members of pair (i, j) take type i's pure properties.
    """
    nt = len(diameters)
    pure = [pure_property(diameters[i], densities[i], youngs_p[i], poisson_p[i]) for i in range(nt)]
    bpp = np.zeros((nt, nt, BP_SIZE))  # [j, i, :] -> record (i, j) at j*nt+i
    for i in range(nt):
        for j in range(nt):
            pari = pure[i]
            parj = pure[i] if quirk_same_type else pure[j]
            bpp[j, i] = binary_property(cf_type, pari, parj, *pp, iswall=False)
    nwt = len(youngs_w)
    walls = [wall_pure_property(youngs_w[w], poisson_w[w]) for w in range(nwt)]
    bpw = np.zeros((nwt, nt, BP_SIZE))
    for i in range(nt):
        for w in range(nwt):
            bpw[w, i] = binary_property(cf_type, pure[i], walls[w], *pw, iswall=True)
    return Tables(radius=np.array([p.radius for p in pure]), mass=np.array([p.mass for p in pure]),
                  inertia=np.array([p.inertia for p in pure]), bpp=bpp.reshape(-1), bpw=bpw.reshape(-1))


def lsd_youngs_for_stiffness(k_n: float, v_ref: float, diameter: float, density: float, poisson: float) -> float:
    """Young's modulus at which the reference's velocity-dependent LSD normal
    stiffness K_n*V**0.4 (Prtcl_ContactForce_inc.f90:24-25) equals k_n at impact
    speed v_ref for two equal spheres; the reference has no direct k_n input."""
    p = pure_property(diameter, density, 1.0, poisson)
    m_eff = p.mass / 2.0
    r_eff = p.radius / 2.0
    coe = k_n / v_ref ** 0.4 / 1.2024
    e_eff = math.sqrt(coe ** 2.5 / (math.sqrt(m_eff) * r_eff))
    return e_eff * 2.0 * (1.0 - poisson * poisson)
