"""Laser envelopes: the initial envelope of a laser pulse, as the reference launches it
(profile_laser_class.f03:319-378 launch, profile_laser_lib.f03 profiles), and the laser
constructor's helpers.

The envelope a = a_r + i a_i of the laser's vector potential is held per xi slice in
azimuthal modes like a 1-component field: arrays ar, ai [nz][P][nr] (P = 2M + 1 mode
parts: m = 0, Re m, Im m; nodes 1..nr).  The perpendicular profiles are the Gaussian beam
and the Laguerre-Gaussian beam; the longitudinal profiles sin^2, the quintic polynomial
(10 t^3 - 15 t^4 + 6 t^5) and the constant.  z is the slice's xi coordinate relative to
the pulse centre, z = (j - 1) dxi + z0 - lon_center; a chirp makes the wavenumber
k = k0 + sum_l c_l z^l.
"""
from __future__ import annotations

import math

import numpy as np


def _laguerre(p: int, alpha: int, x: float) -> float:
    """Generalised Laguerre polynomial L_p^alpha(x) by its three-term recurrence."""
    if p == 0:
        return 1.0
    l0, l1 = 1.0, 1.0 + alpha - x
    for k in range(1, p):
        l0, l1 = l1, ((2 * k + 1 + alpha - x) * l1 - (k + alpha) * l0) / (k + 1)
    return l1


def gaussian(r, z, k, k0, w0, f_dist, mode):
    """get_prof_perp_gaussian (profile_laser_lib.f03:56-96): (ar_re, ar_im, ai_re, ai_im)."""
    if mode != 0:
        return 0.0, 0.0, 0.0, 0.0
    z_shift = -1.0 * (z + f_dist)
    r2 = r * r
    z2 = z_shift * z_shift
    zr = 0.5 * k * w0 * w0
    zr2 = zr * zr
    curv = z_shift / (z2 + zr2)
    w = w0 * math.sqrt(1.0 + z2 / zr2)
    gouy = math.atan2(z_shift, zr)
    phase = 0.5 * k * r2 * curv - gouy - (k - k0) * z
    amp = w0 / w * math.exp(-r2 / (w * w))
    return amp * math.cos(phase), 0.0, -amp * math.sin(phase), 0.0


def laguerre(r, z, k, k0, w0, f_dist, radial_index, phi_index, mode):
    """get_prof_perp_laguerre (profile_laser_lib.f03:122-190): the (p, l) Laguerre-Gaussian
    beam in mode l, OSIRIS normalisation."""
    p, l = radial_index, phi_index
    if mode != l:
        return 0.0, 0.0, 0.0, 0.0
    z_shift = -1.0 * (z + f_dist)
    r2 = r * r
    z2 = z_shift * z_shift
    zr = 0.5 * k * w0 * w0
    zr2 = zr * zr
    curv = z_shift / (z2 + zr2)
    w2 = w0 * w0 * (1.0 + z2 / zr2)
    r2_iw2 = r2 / w2
    gouy = float(1 + 2 * p + abs(l)) * math.atan2(z_shift, zr)
    phase = 0.5 * k * r2 * curv - gouy - (k - k0) * z
    amp = w0 / math.sqrt(w2) * math.exp(-r2_iw2) * math.sqrt(r2_iw2) ** abs(l) * _laguerre(p, abs(l), 2.0 * r2_iw2)
    if mode == 0:
        return amp * math.cos(phase), amp * math.sin(phase), 0.0, 0.0
    ar_re, ar_im = 0.5 * amp * math.cos(phase), 0.5 * amp * math.sin(phase)
    return ar_re, ar_im, -ar_im, ar_re


def longitudinal(z, lon) -> float:
    """get_prof_lon_sin2 / _poly / get_prof_const (profile_laser_lib.f03:440-554):
    lon = ("sin2" | "poly", t_rise, t_flat, t_fall) or ("const",)."""
    kind = lon[0]
    if kind == "const":
        return 1.0
    t_rise, t_flat, t_fall = lon[1], lon[2], lon[3]
    fs, fe = -0.5 * t_flat, 0.5 * t_flat
    if z < fs - t_rise or z >= fe + t_fall:
        return 0.0
    if fs <= z < fe:
        return 1.0
    if kind == "sin2":
        e = math.cos((z - fs) / t_rise * (0.5 * math.pi)) if z < fs else math.cos((z - fe) / t_fall * (0.5 * math.pi))
        return e * e
    if kind == "poly":
        t = (z + t_rise - fs) / t_rise if z < fs else (fe + t_fall - z) / t_fall
        return 10.0 * t ** 3 - 15.0 * t ** 4 + 6.0 * t ** 5
    raise ValueError(f"unknown longitudinal profile {kind!r}")


def launch(nr, nz, max_mode, dr, dxi, *, k0, a0, w0, focal_distance=0.0, lon=("const",), lon_center=0.0,
           z0=0.0, chirp_coefs=(0.0,), profile="gaussian", radial_index=0, phi_index=0):
    """launch_profile_laser (profile_laser_class.f03:319-378): the initial envelope
    (ar, ai), each [nz][P][nr]."""
    P = 2 * max_mode + 1
    ar = np.zeros((nz, P, nr))
    ai = np.zeros((nz, P, nr))
    for j in range(1, nz + 1):
        z = (j - 1) * dxi + z0 - lon_center
        k = k0
        for l, c in enumerate(chirp_coefs, start=1):
            k = k + c * z ** l
        env = longitudinal(z, lon) * a0
        for m in range(max_mode + 1):
            for i in range(1, nr + 1):
                r = (i - 1) * dr
                if profile == "gaussian":
                    arr, ari, air, aii = gaussian(r, z, k, k0, w0, focal_distance, m)
                elif profile == "laguerre":
                    arr, ari, air, aii = laguerre(r, z, k, k0, w0, focal_distance, radial_index, phi_index, m)
                else:
                    raise ValueError(f"unknown perpendicular profile {profile!r}")
                if m == 0:
                    ar[j - 1, 0, i - 1] = env * arr
                    ai[j - 1, 0, i - 1] = env * air
                else:
                    ar[j - 1, 2 * m - 1, i - 1] = env * arr
                    ai[j - 1, 2 * m - 1, i - 1] = env * air
                    ar[j - 1, 2 * m, i - 1] = env * ari
                    ai[j - 1, 2 * m, i - 1] = env * aii
    return ar, ai
