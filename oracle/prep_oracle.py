"""ORACLE — test infrastructure, never the product.

CPU restatement of the reference's input preprocessors for one rank, in numpy float32 /
Python float (double) scalar arithmetic in the reference's order:

* read_grid_coord (code/srcF/seis3d_grid.F90:89-149): uniform or listed axes, degrees to
  radians, distance2meter, linear ghost extrapolation;
* io_pt_read (code/srcF/mod_io.F90:112-152) and receiver_locate
  (code/srcF/seis3d_station.F90:64-105);
* read_src_para, angle2moment and the source locating loops
  (code/srcF/seis3d_source.F90:60-160, 324-425).

Only the tests use it, as the checker of the `fwant_prep` program.  Parity is pinned to
this restatement alone: the reference ships no input files or outputs for these programs.
"""
from __future__ import annotations

import math

import numpy as np

LENFD = 3
SEIS_ZERO = np.float32(1.0e-20)
f32 = np.float32


def grid_axis(n: int, dh: float, x0: float, values=None, top: bool = False, degrees: bool = True,
              d2m: float = 1.0) -> np.ndarray:
    """One axis of read_grid_coord with its 3 ghosts on each side (seis3d_grid.F90:107-147)."""
    nx = n + 2 * LENFD
    i1, i2 = LENFD, LENFD + n - 1
    g = [f32(0.0)] * nx
    dh, x0 = f32(dh), f32(x0)
    if dh >= SEIS_ZERO:
        for q in range(nx):
            idx = q - nx + 1 + LENFD if top else q - i1   # (k-num_z+LenFD) or (i-ni1)
            g[q] = f32(f32(idx) * dh) + x0
    else:
        v = np.asarray(values, np.float32)
        assert v.size == n
        for q in range(n):
            g[i1 + q] = f32(v[q])
    if degrees:
        g = [f32(float(v) / 180.0 * math.pi) for v in g]      # gx/180.0_DP*PI
    else:
        g = [f32(v * f32(d2m)) for v in g]                   # gz*d2m
    for q in range(1, LENFD + 1):
        g[i1 - q] = f32(f32(g[i1 - q + 1] + g[i1]) - g[i1 + 1])
        g[i2 + q] = f32(f32(g[i2 + q - 1] + g[i2]) - g[i2 - 1])
    return np.array(g, np.float32)


def _deg2rad(v) -> np.float32:
    """real(SP) * PI / 180 in double, stored in SP (pt_xyz(1:2,:)*PI/180.0_SP)."""
    return f32(float(f32(v)) * math.pi / 180.0)


def _minloc_abs(a: np.ndarray, v) -> int:
    """minloc(abs(a - v)), 1-based, first minimum wins."""
    a = np.asarray(a, np.float32)
    d = np.abs(a - f32(v))
    return int(np.argmin(d)) + 1


def station_points(recvs, lines):
    """io_pt_read: receivers (x, y, z) then each line (x0, y0, z0, dx, dy, dz, npt) as points
    x0 + dx*(m-1); theta and phi from degrees.  Returns xyz (npt, 3) float32 and id (npt, 2)."""
    xyz, ids = [], []
    for n, r in enumerate(recvs, start=1):
        xyz.append([f32(v) for v in r])
        ids.append((n, 0))
    for n, ln in enumerate(lines, start=1):
        x0 = [f32(v) for v in ln[0:3]]
        dx = [f32(v) for v in ln[3:6]]
        for m in range(1, int(ln[6]) + 1):
            xyz.append([f32(x0[d] + f32(dx[d] * f32(m - 1))) for d in range(3)])
            ids.append((m, n))
    for p in xyz:
        p[0], p[1] = _deg2rad(p[0]), _deg2rad(p[1])
    return np.array(xyz, np.float32).reshape(-1, 3), np.array(ids, np.int32).reshape(-1, 2)


def receiver_locate(xyz, ids, x, y, z, ni, nj, nk, topo_hyper_height):
    """Nearest node of every point; points above topo_hyper_height go to the free surface
    k = nk2; points whose node is a ghost are dropped.  Returns the station file's
    variables (indx, gindx, coord, grid, id), one row per kept point."""
    out = {k: [] for k in ("indx", "gindx", "coord", "grid", "id")}
    nk2 = nk + LENFD
    for p, pid in zip(xyz, ids):
        x0, y0, z0 = f32(p[0]), f32(p[1]), f32(p[2])
        i, j = _minloc_abs(x, x0), _minloc_abs(y, y0)
        k = _minloc_abs(z, z0) if z0 <= f32(topo_hyper_height) else nk2
        if not (LENFD < i <= ni + LENFD and LENFD < j <= nj + LENFD and LENFD < k <= nk2):
            continue
        out["indx"].append((i, j, k))
        out["gindx"].append((i - LENFD, j - LENFD, k - LENFD))
        out["coord"].append((x0, y0, z0))
        out["grid"].append((x[i - 1], y[j - 1], z[k - 1]))
        out["id"].append(tuple(pid))
    return {k: np.array(v, np.float32 if k in ("coord", "grid") else np.int32).reshape(-1, 2 if k == "id" else 3)
            for k, v in out.items()}


def angle2moment(strike: float, dip: float, rake: float):
    """Aki & Richards double couple in double, each component rounded to SP, as spherical
    (Mxx, Myy, Mzz, Mxy, Mxz, Myz) (seis3d_source.F90:403-425)."""
    d, s, r = dip / 180.0 * math.pi, strike / 180.0 * math.pi, rake / 180.0 * math.pi
    sin, cos = math.sin, math.cos
    m11 = f32(-(sin(d) * cos(r) * sin(2.0 * s) + sin(2.0 * d) * sin(r) * (sin(s) * sin(s))))
    m22 = f32(sin(d) * cos(r) * sin(2.0 * s) - sin(2.0 * d) * sin(r) * (cos(s) * cos(s)))
    m33 = f32(-f32(m11 + m22))
    m12 = f32(sin(d) * cos(r) * cos(2.0 * s) + 0.5 * sin(2.0 * d) * sin(r) * sin(2.0 * s))
    m13 = f32(-(cos(d) * cos(r) * cos(s) + cos(2.0 * d) * sin(r) * sin(s)))
    m23 = f32(-(cos(d) * cos(r) * sin(s) - cos(2.0 * d) * sin(r) * cos(s)))
    return [m11, m22, m33, f32(-m12), m13, f32(-m23)]


def forces(records, ntw):
    """read_src_para's force records, ntw per source: (x, y, z, t0, f0, fx, fy, fz); the
    components are scaled by f0 in SP.  Returns axis (n, 3), t0 (n), F (3, n, ntw)."""
    n = len(records) // ntw
    axis = np.zeros((n, 3), np.float32)
    t0 = np.zeros(n, np.float32)
    F = np.zeros((3, n, ntw), np.float32)
    for q in range(n):
        for m in range(ntw):
            r = [f32(v) for v in records[q * ntw + m]]
            axis[q] = r[0:3]
            t0[q] = r[3]
            for c in range(3):
                F[c, q, m] = f32(r[5 + c] * r[4])
        axis[q, 0], axis[q, 1] = _deg2rad(axis[q, 0]), _deg2rad(axis[q, 1])
    return axis, t0, F


def moments(records, ntw, mech: str):
    """read_src_para's moment records: (x, y, z, t0, m0, Mxx, Myy, Mzz, Mxy, Mxz, Myz) for
    mech 'moment', else (x, y, z, t0, m0, strike, dip, rake) with strike, dip and rake read
    as double.  Returns axis (n, 3), t0 (n), M (6, n, ntw)."""
    n = len(records) // ntw
    axis = np.zeros((n, 3), np.float32)
    t0 = np.zeros(n, np.float32)
    M = np.zeros((6, n, ntw), np.float32)
    for q in range(n):
        for m in range(ntw):
            rec = records[q * ntw + m]
            axis[q] = [f32(v) for v in rec[0:3]]
            t0[q] = f32(rec[3])
            m0 = f32(rec[4])
            t = [f32(v) for v in rec[5:11]] if mech == "moment" else angle2moment(*[float(v) for v in rec[5:8]])
            for c in range(6):
                M[c, q, m] = f32(m0 * t[c])
        axis[q, 0], axis[q, 1] = _deg2rad(axis[q, 0]), _deg2rad(axis[q, 1])
    return axis, t0, M


def locate_sources(axis, x, y, z, ni, nj, nk, src_hyper_height):
    """Nearest node and fractional shift of each source (seis3d_source.F90:60-160).  A
    source above the grid and above src_hyper_height goes to k = nk2 at the surface radius.
    Returns indx (n, 3), axis (n, 3) with z updated, shift (n, 3) and found (n)."""
    axis = np.array(axis, np.float32).reshape(-1, 3).copy()
    n = axis.shape[0]
    indx = np.zeros((n, 3), np.int32)
    shift = np.zeros((n, 3), np.float32)
    found = np.zeros(n, bool)
    x, y, z = (np.asarray(a, np.float32) for a in (x, y, z))
    nk2 = nk + LENFD

    def sh(a, i, v):
        c = a[i - 1]
        return f32(f32(v - c) / f32(a[i] - c)) if v > c else f32(f32(v - c) / f32(c - a[i - 2]))

    for q in range(n):
        x0, y0, z0 = axis[q]
        if x0 < x.min() or x0 > x.max() or y0 < y.min() or y0 > y.max():
            continue
        i, j = _minloc_abs(x, x0), _minloc_abs(y, y0)
        if z.min() <= z0 <= z.max():
            k = _minloc_abs(z, z0)
        elif z0 > f32(src_hyper_height):
            k = nk2
            z0 = z[k - 1]
        else:
            continue
        if not (LENFD < i <= ni + LENFD and LENFD < j <= nj + LENFD and LENFD < k <= nk2):
            continue
        found[q] = True
        indx[q] = (i, j, k)
        axis[q, 2] = z0
        shift[q] = (sh(x, i, x0), sh(y, j, y0), sh(z, k, z0))
    return indx, axis, shift, found
