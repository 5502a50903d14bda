"""Seeded models of the terrain-following (Gaussian-hill) extension shared by the CPU and
GPU tests.  The extension has no counterpart in the reference: its grid is orthogonal
spherical with a flat top (code/srcF/mod_grid.F90:36-38, seis3d_metric.F90:83-112)."""
import numpy as np

from fwant_gb300 import inputs

LENFD = 3


def hill_model(ni=40, nj=40, nk=30, amp=2000.0, width_km=8.0, kind="surface", seed=3):
    """A small model with a 2 km Gaussian hill centred on the surface source column,
    8-cell PML on five faces, free surface, eight seeded surface receivers plus two on the
    hill's flank."""
    if kind == "surface":
        m = inputs.make_model(ni, nj, nk, seed=seed, npml=8, nrecv=8, source="surface", fc=0.3, t0=4.0)
    else:
        m = inputs.make_model(ni, nj, nk, seed=seed, npml=8, nrecv=8, source="buried", fc=0.3, t0=4.0,
                              force=(3.0e14, -2.0e14, 1.0e15))
    c = (LENFD + ni // 2 + 1, LENFD + nj // 2 + 1)
    flank = np.array([[c[0] + 4, c[1] - 3, nk + LENFD], [c[0] - 6, c[1] + 2, nk + LENFD]], np.int32)
    m.recv_indx = np.concatenate([m.recv_indx, flank]).astype(np.int32)
    h = inputs.gaussian_hill(m, amp, width_km, centre=c)
    return m, h


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


def convergence_level(level, base=(48, 48, 24), amp=2000.0, width_km=8.0, fc=0.15, t0=8.0, dt0=0.05):
    """Level l of the self-convergence study on the hill: uniform spacing 1 km / 2^l in
    all three directions over the same 48 x 48 x 24 km box (nodes of level 0 stay nodes),
    8 * 2^l PML cells on five faces, a vertical surface force on the hill top, time step
    dt0 / 2^l; receivers at four surface nodes of level 0 on the hill."""
    f = 2 ** level
    ni, nj, nk = base[0] * f, base[1] * f, base[2] * f
    m = inputs.make_model(ni, nj, nk, seed=1, dh_km=1.0 / f, z_top_km=1.0 / f, z_bottom_km=1.0 / f, npml=8 * f,
                          nrecv=0, source="surface", fc=fc, t0=t0)
    ic, jc = LENFD + ni // 2 + 1, LENFD + nj // 2 + 1
    m.force_indx = np.array([[ic, jc, nk + LENFD]], np.int32)
    m.stept = float(np.float32(dt0 / f))
    offs = ((4, 0), (0, -6), (-5, 5), (8, 8))
    m.recv_indx = np.array([[ic + a * f, jc + b * f, nk + LENFD] for a, b in offs], np.int32)
    h = inputs.gaussian_hill(m, amp, width_km, centre=(ic, jc))
    return m, h
