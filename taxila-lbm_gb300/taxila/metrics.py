"""Derived quantities of a flow state, used to state the error of the
reduced-precision forms against the FP64 oracle.

All functions take natural-order fields as returned by tx_download (component
fastest) and the lattice shape (nz, ny, nx).
"""
import numpy as np


def permeability(tau, gz, flux, walls, nsites):
    """k = nu <u_z>_pore phi / g for single-phase flow driven by a body force
    g along z, with nu = (tau - 1/2) / 3 and <u_z>_pore phi = sum of u_z over
    pore sites / all sites (lattice units)."""
    u = np.asarray(flux).reshape(nsites, -1)
    pore = np.asarray(walls).ravel() == 0
    return (tau - 0.5) / 3.0 * (u[pore, -1].sum() / nsites) / gz


def phase_fraction(rho, ncomp, comp, lo, hi):
    """Fraction of each site occupied by component ``comp`` between its two
    bulk densities lo (absent) and hi (present), clipped to [0, 1]."""
    r = np.asarray(rho).reshape(-1, ncomp)[:, comp]
    return np.clip((r - lo) / (hi - lo), 0.0, 1.0)


def equivalent_radius(rho, ncomp, comp, lo, hi, ndims):
    """Radius of the disk (2D) or sphere (3D) with the volume of component
    ``comp``'s phase: the interface position of a bubble."""
    v = phase_fraction(rho, ncomp, comp, lo, hi).sum()
    return np.sqrt(v / np.pi) if ndims == 2 else (3.0 * v / (4.0 * np.pi)) ** (1.0 / 3.0)


def front_position(rho, shape, ncomp, comp, lo, hi, walls):
    """Mean z of the invading component's front: the saturation-weighted
    penetration depth, sum over pore sites of the phase fraction divided by the
    pore area of a z slice (lattice units from z = 0)."""
    nz, ny, nx = shape
    s = phase_fraction(rho, ncomp, comp, lo, hi).reshape(shape)
    pore = (np.asarray(walls).ravel() == 0).reshape(shape)
    area = pore.sum(axis=(1, 2)).astype(float)
    filled = (s * pore).sum(axis=(1, 2))
    return float(np.sum(np.divide(filled, area, out=np.zeros_like(filled), where=area > 0)))


def saturation(rho, ncomp, comp, lo, hi, walls):
    """Pore-volume fraction occupied by component ``comp``."""
    pore = np.asarray(walls).ravel() == 0
    return float(phase_fraction(rho, ncomp, comp, lo, hi)[pore].mean())


def rel_err(a, b, mask=None):
    """max |a - b| / max |b| (over mask)."""
    a, b = np.asarray(a), np.asarray(b)
    if mask is not None:
        a, b = a[mask], b[mask]
    return float(np.max(np.abs(a - b)) / (np.max(np.abs(b)) or 1.0))
