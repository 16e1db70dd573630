"""Mie series for a homogeneous sphere in vacuum: the independent physics
oracle for the scattered and absorbed power of the sphere workloads.

TEST INFRASTRUCTURE ONLY (tests/, smoke() and the bench's accuracy report).

Restates the published Lorenz-Mie solution (Bohren & Huffman, "Absorption and
Scattering of Light by Small Particles", eqs. 4.53, 4.61, 4.62), non-magnetic
sphere (mu = 1), in the reference's units: lengths in microns, angular
frequency omega in units of 3e14 rad/s (so k0 = omega), incident field of unit
amplitude, power = cross section * |E0|^2 / (2 ZVAC) in watts
(libs/libscuff/libscuff.h:77-79 for ZVAC; the same convention as the Mie
tables of unitTests/unit-test-PFT.cc:60-130, which pin this module).
"""
from __future__ import annotations

import numpy as np
from scipy.special import spherical_jn, spherical_yn

ZVAC = 376.73031346177


def _riccati(n, z):
    """psi_n(z) = z j_n(z) and its derivative, for complex or real z."""
    j = spherical_jn(n, z)
    dj = spherical_jn(n, z, derivative=True)
    return z * j, j + z * dj


def _riccati_h(n, x):
    """xi_n(x) = x h_n^(1)(x) and its derivative (real x)."""
    h = spherical_jn(n, x) + 1j * spherical_yn(n, x)
    dh = spherical_jn(n, x, derivative=True) + 1j * spherical_yn(n, x, derivative=True)
    return x * h, h + x * dh


def coefficients(omega, radius=1.0, eps=None, pec=False, nmax=None):
    """Mie coefficients a_n, b_n (n = 1..nmax) of a sphere of permittivity eps
    (complex, relative) or a perfect conductor (pec=True) at size parameter
    x = omega * radius."""
    x = float(omega) * float(radius)
    if nmax is None:
        nmax = int(x + 4.0 * x ** (1.0 / 3.0) + 8)
    n = np.arange(1, nmax + 1)
    psi_x, dpsi_x = _riccati(n, x)
    xi_x, dxi_x = _riccati_h(n, x)
    if pec:
        return dpsi_x / dxi_x, psi_x / xi_x
    m = np.sqrt(complex(eps))
    psi_m, dpsi_m = _riccati(n, m * x)
    a = (m * psi_m * dpsi_x - psi_x * dpsi_m) / (m * psi_m * dxi_x - xi_x * dpsi_m)
    b = (psi_m * dpsi_x - m * psi_x * dpsi_m) / (psi_m * dxi_x - m * xi_x * dpsi_m)
    return a, b


def cross_sections(omega, radius=1.0, eps=None, pec=False):
    """(sigma_abs, sigma_sca) in square microns."""
    a, b = coefficients(omega, radius, eps, pec)
    x = float(omega) * float(radius)
    n = np.arange(1, len(a) + 1)
    geo = np.pi * radius ** 2
    qsca = 2.0 / x ** 2 * np.sum((2 * n + 1) * (np.abs(a) ** 2 + np.abs(b) ** 2))
    qext = 2.0 / x ** 2 * np.sum((2 * n + 1) * np.real(a + b))
    return (qext - qsca) * geo, qsca * geo


def powers(omega, radius=1.0, eps=None, pec=False, e0=1.0):
    """(absorbed, scattered) power in watts for an incident field of
    amplitude |E0| = e0 (V/micron)."""
    sa, ss = cross_sections(omega, radius, eps, pec)
    f = abs(e0) ** 2 / (2.0 * ZVAC)
    return sa * f, ss * f
