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


def convergence_level(level, base=(48, 48, 24), amp=2000.0, width_km=8.0, fc=0.15, t0=8.0, dt0=0.05,
                      vp=6000.0, vs=6000.0 / 1.73, rho=2700.0, depth_km=6):
    """Level l of the self-convergence study on the hill: the same 48 x 48 x 24 km box at
    uniform spacing 1 km / 2^l in all three directions (base * 2^l + 1 nodes, so level-0
    nodes stay nodes), a homogeneous medium (Vp 6 km/s, Vs = Vp / 1.73, 2700 kg/m^3), so
    that every level discretises the same physical model, 8 * 2^l PML cells (8 km) on five
    faces, time step dt0 / 2^l (CFL 0.3); receivers at four surface nodes of level 0 on the
    hill's flanks.  The vertical force sits depth_km below the hill top (the node
    depth_km * 2^l planes under the surface, at the same point of the terrain-following
    grid at every level; its 7^3 smoothing stays clear of the free surface); depth_km = 0
    puts it on the surface, where the reference's traction source converges only to first
    order (the flat top shows the same 24% difference between 1 and 0.5 km)."""
    f = 2 ** level
    ni, nj, nk = base[0] * f + 1, base[1] * f + 1, base[2] * f + 1
    m = inputs.make_model(ni, nj, nk, seed=1, dh_km=1.0 / f, z_top_km=1.0 / f, z_bottom_km=1.0 / f, npml=8 * f,
                          nrecv=0, source="surface", fc=fc, t0=t0)
    shape = m.lam.shape
    mu = rho * vs * vs
    m.lam = np.full(shape, rho * vp * vp - 2.0 * mu, np.float32, order="F")
    m.mu = np.full(shape, mu, np.float32, order="F")
    m.rho = np.full(shape, rho, np.float32, order="F")
    ic, jc = LENFD + (ni - 1) // 2 + 1, LENFD + (nj - 1) // 2 + 1
    m.force_indx = np.array([[ic, jc, nk + LENFD - depth_km * f]], np.int32)
    m.stept = float(np.float32(dt0 / f))
    offs = ((4, 0), (0, -6), (-5, 5), (8, 8))
    m.recv_indx = np.array([[ic + a * f, jc + b * f, nk + LENFD] for a, b in offs], np.int32)
    h = inputs.gaussian_hill(m, amp, width_km, centre=(ic, jc))
    return m, h
