"""Neutral gas species: ADK ionisation rate coefficients and the species constructor.

The reference compiles a table of per-level rate coefficients for a list of elements
(neutral_class.f03:18-350) and evaluates the ADK tunnelling rate of level i as
    w_i(E) = p1_i E^(-p3_i) exp(-p2_i / E)    (w in 1/s, E in GV/m).
Here the caller passes (p1, p2, p3) per level; `adk_coefficients` derives them from the
levels' ionisation energies with the ADK formula for l = m = 0 (M. V. Ammosov, N. B.
Delone, V. P. Krainov, Sov. Phys. JETP 64, 1191 (1986)), in atomic units:
    w = omega_a C^2 U (2 (2U)^(3/2) E_a / E)^(2 n* - 1) exp(-2 (2U)^(3/2) E_a / (3 E)),
    n* = Z / sqrt(2 U),  C^2 = 2^(2 n*) / (n* Gamma(n* + 1) Gamma(n*)),
with U the ionisation energy in hartree, Z the charge after ionisation, omega_a the atomic
unit of frequency and E_a the atomic unit of field.  Hence p2 = 2 (2U)^(3/2) E_a / 3,
p3 = 2 n* - 1 and p1 = omega_a C^2 U (2 (2U)^(3/2) E_a)^(2 n* - 1).
"""
from __future__ import annotations

import math

HARTREE_EV = 27.211386245988          # hartree in eV
OMEGA_A = 4.1341373335e16             # atomic unit of frequency (1/s)
E_A_GVM = 514.22067476                # atomic unit of field (GV/m)


def adk_coefficients(energies_ev) -> list:
    """[(p1, p2, p3)] per ionisation level from the levels' ionisation energies (eV)."""
    out = []
    for k, u_ev in enumerate(energies_ev):
        U = u_ev / HARTREE_EV
        Z = k + 1
        ns = Z / math.sqrt(2.0 * U)
        c2 = 2.0 ** (2.0 * ns) / (ns * math.gamma(ns + 1.0) * math.gamma(ns))
        f = 2.0 * (2.0 * U) ** 1.5 * E_A_GVM
        out.append((OMEGA_A * c2 * U * f ** (2.0 * ns - 1.0), f / 3.0, 2.0 * ns - 1.0))
    return out


def plasma_frequency(n0_cm3: float) -> float:
    """Electron plasma frequency (1/s) of a density in cm^-3."""
    return 5.641460e4 * math.sqrt(n0_cm3)
