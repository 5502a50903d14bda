"""Physics checks of the forward solver that a faithful restatement cannot pass by
construction: source-receiver reciprocity for surface forces, energy decay once the
wavefield has entered the CFS-PML, and the convergence order under grid refinement.

Each experiment takes a factory ``make(ni, nj, nk, stept, free_surface)`` that returns a
solver object with the set-up methods of ``fwant_gb300.Solver`` (the oracle's ``Oracle``
has the same ones), so the same checks run on the CPU restatement and on the GPU.

References for the physics being checked:
* surface forces: src_surface, code/srcF/mod_src.F90:373-414; receivers: io_seismo_put,
  code/srcF/mod_io.F90:461-497;
* the CFS-PML: abs_L<X> and abs_RK_*, code/srcF/mod_abs_npml.F90:641-2123;
* the DRP/opt MacCormack operators, code/srcF/mod_macdrp.h:19-103, inside classical RK4
  (mod_macdrp.F90:291-393).
"""
from __future__ import annotations

import numpy as np

from fwant_gb300 import inputs

LENFD = 3


# ---- reciprocity ---------------------------------------------------------------------------
def reciprocity_model(seed=5, z_top_km=0.5, z_bottom_km=2.0, nk=28):
    """44 x 40 x nk cells of the C2 physics (1 km horizontal, vertical spacing from
    z_top_km at the surface to z_bottom_km, +/-5% Gaussian-correlated perturbation, 8-cell
    CFS-PML on five faces, free surface, 0.2 Hz Ricker centred at 6 s) and two surface
    stations A and B about 15 km apart, not mirror images of each other.  Returns the
    model, A, B and the number of steps covering 18 s."""
    m = inputs.make_model(44, 40, nk, seed=seed, npml=8, nrecv=0, perturb=0.05, source="surface", fc=0.2, t0=6.0,
                          z_top_km=z_top_km, z_bottom_km=z_bottom_km)
    ic, jc, kc = LENFD + m.ni // 2 + 1, LENFD + m.nj // 2 + 1, m.nk + LENFD
    a = (ic - 7, jc - 3, kc)
    b = (ic + 6, jc + 4, kc)
    return m, a, b, int(18.0 / m.stept) + 1


def reciprocity_gathers(make, m, a, b, nsteps):
    """Velocity Green's functions between the stations: g[(s, r)][i, j] is the trace of
    velocity component i at station r for a unit-direction force j (1e15 N) at station s."""
    out = {}
    for src, rcv in ((a, b), (b, a)):
        for j in range(3):
            s = make(m.ni, m.nj, m.nk, m.stept, True)
            f = [np.zeros((1, 1), np.float32) for _ in range(3)]
            f[j][0, 0] = np.float32(1.0e15)
            inputs.attach(s, m)
            s.set_forces(np.array([src], np.int32), np.zeros((1, 3), np.float32), np.zeros(1, np.float32),
                         m.stf_time, m.stf_freq, f[0], f[1], f[2], 200)
            s.set_receivers(np.array([rcv], np.int32), 1)
            s.run(nsteps)
            g = s.get_seismo()          # (9, nsamp, 1)
            out.setdefault((src, rcv), np.zeros((3, 3, g.shape[1])))[:, j, :] = g[:3, :, 0]
            if hasattr(s, "close"):
                s.close()
    return out


def reciprocity_errors(g, a, b, floor=0.05):
    """Relative L2 difference of G_ij(A <- B) and G_ji(B <- A) for every (i, j) pair whose
    trace is at least `floor` of the largest trace norm (weaker pairs are rounding-level
    in a nearly layered medium)."""
    gab, gba = g[(b, a)], g[(a, b)]   # gab[i, j]: at A from force j at B
    norms = np.sqrt(np.sum(gab ** 2, axis=-1))
    big = norms.max()
    errs = {}
    for i in range(3):
        for j in range(3):
            x, y = gab[i, j], gba[j, i]
            n = max(np.sqrt(np.sum(x * x)), np.sqrt(np.sum(y * y)))
            if n < floor * big:
                continue
            errs[("xyz"[i], "xyz"[j])] = float(np.sqrt(np.sum((x - y) ** 2)) / n)
    return errs


# ---- energy in the PML ---------------------------------------------------------------------
def energy_model(npml, seed=9):
    """40 x 40 x 30 cells, layered medium, free surface, a buried oblique force with a
    0.3 Hz Ricker wavelet centred at 4 s; CFS-PML of npml cells on five faces (0: none,
    the zero ghost values then reflect)."""
    return inputs.make_model(40, 40, 30, seed=seed, npml=npml, nrecv=0, source="buried", fc=0.3, t0=4.0,
                             force=(5.0e14, -3.0e14, 1.0e15))


def energy(s, m, margin):
    """Elastic energy in the cells at least `margin` cells from the four side faces and the
    bottom (outside any PML slab): sum over points of
    (rho |v|^2 / 2 + (sigma:sigma - lambda/(3 lambda + 2 mu) tr(sigma)^2) / (4 mu)) dV,
    dV = r^2 sin(theta) dr dtheta dphi."""
    sl = (slice(LENFD + margin, LENFD + m.ni - margin), slice(LENFD + margin, LENFD + m.nj - margin),
          slice(LENFD + margin, LENFD + m.nk))
    f = [np.asarray(s.get_field(c), np.float64)[sl] for c in range(9)]
    vx, vy, vz, txx, tyy, tzz, txy, txz, tyz = f
    lam = m.lam[sl].astype(np.float64)
    mu = m.mu[sl].astype(np.float64)
    rho = m.rho[sl].astype(np.float64)
    kin = 0.5 * rho * (vx * vx + vy * vy + vz * vz)
    ss = txx ** 2 + tyy ** 2 + tzz ** 2 + 2 * (txy ** 2 + txz ** 2 + tyz ** 2)
    tr = txx + tyy + tzz
    strain = (ss - lam / (3 * lam + 2 * mu) * tr * tr) / (4 * mu)
    x, y, z = (np.asarray(v, np.float64) for v in (m.x, m.y, m.z))
    dx = np.gradient(x)[sl[0]]
    dy = np.gradient(y)[sl[1]]
    dz = np.gradient(z)[sl[2]]
    dv = (dx * np.sin(x[sl[0]]))[:, None, None] * dy[None, :, None] * (z[sl[2]] ** 2 * dz)[None, None, :]
    return float(np.sum((kin + strain) * dv))


def energy_history(make, m, margin, nsteps, every):
    s = make(m.ni, m.nj, m.nk, m.stept, True)
    inputs.attach(s, m)
    t, e = [], []
    for n in range(0, nsteps, every):
        s.run(every)
        t.append((n + every) * m.stept)
        e.append(energy(s, m, margin))
    if hasattr(s, "close"):
        s.close()
    return np.array(t), np.array(e)


# ---- convergence order ---------------------------------------------------------------------
VP, VS, RHO = 6000.0, 6000.0 / 1.73, 2700.0


def convergence_grid(level, size_km=48.0, h0_km=1.0, theta_c_deg=50.0, phi_c_deg=100.0):
    """Uniform spherical grid of a size_km cube at spacing h0_km / 2^level: colatitude and
    longitude steps h / R_top, radial step h, top at R_top.  Returns n and float64 node
    coordinates with ghosts (theta, phi in rad, r in m).  The cube is wide enough (48 km
    for the 4 km pulse run to 0.8 s) that the field stays below 1e-8 of its peak at the
    faces, whose zero ghost values would otherwise add an error that does not shrink with
    the spacing (a 32 km cube stalls at a 7e-4 difference from the 0.25 km level on)."""
    h = h0_km / 2 ** level
    n = int(round(size_km / h)) + 1  # node-centred refinement: level-0 nodes stay nodes
    R = inputs.R_EARTH_KM * 1000.0
    dang = h * 1000.0 / R
    idx = np.arange(n + 2 * LENFD) - LENFD
    th = np.deg2rad(theta_c_deg) + (idx - (n - 1) / 2.0) * dang
    ph = np.deg2rad(phi_c_deg) + (idx - (n - 1) / 2.0) * dang
    r = R + (idx - (n - 1)) * h * 1000.0
    return n, th, ph, r, h * 1000.0, dang


def convergence_solution(make, level, t_end=0.8, steps0=16, width_km=4.0):
    """Initial-value problem in a homogeneous medium (Vp 6 km/s, Vs = Vp/1.73, rho 2700):
    an isotropic stress pulse sigma_ii = 1e6 exp(-d^2/w^2) Pa at the cube's centre, no
    source, no PML, no free surface, run to t_end with steps0 * 2^level steps (CFL 0.3 at
    every level).  The metric is the exact one of the uniform grid (1/dtheta, 1/dphi,
    1/dr, sin and cot of the colatitude in double), so that FP32 coordinate rounding
    does not enter.  Returns the nine fields on the interior, float64."""
    n, th, ph, r, dr, dang = convergence_grid(level)
    nsteps = steps0 * 2 ** level
    stept = t_end / nsteps
    s = make(n, n, n, stept, False)
    s.set_coord(th.astype(np.float32), ph.astype(np.float32), r.astype(np.float32))
    nx = n + 2 * LENFD
    s.set_metric(np.sin(th).astype(np.float32), (1.0 / np.tan(th)).astype(np.float32),
                 np.full(nx, 1.0 / dang, np.float32), np.full(nx, 1.0 / dang, np.float32),
                 np.full(nx, 1.0 / dr, np.float32))
    shape = (nx, nx, nx)
    mu = RHO * VS * VS
    lam = RHO * VP * VP - 2 * mu
    s.set_media(np.full(shape, lam, np.float32, order="F"), np.full(shape, mu, np.float32, order="F"),
                np.full(shape, RHO, np.float32, order="F"))
    s.set_pml(np.zeros(6, np.int32), np.zeros(6, np.float32), np.ones(6, np.float32), np.zeros(6, np.float32))
    T, P, R = np.meshgrid(th, ph, r, indexing="ij")
    X, Y, Z = R * np.sin(T) * np.cos(P), R * np.sin(T) * np.sin(P), R * np.cos(T)
    c = nx // 2
    d2 = (X - X[c, c, c]) ** 2 + (Y - Y[c, c, c]) ** 2 + (Z - Z[c, c, c]) ** 2
    p = np.asfortranarray((1.0e6 * np.exp(-d2 / (width_km * 1000.0) ** 2)).astype(np.float32))
    for comp in ("Txx", "Tyy", "Tzz"):
        s.set_field(comp, p)
    s.run(nsteps)
    out = np.stack([np.asarray(s.get_field(q), np.float64)[LENFD:-LENFD, LENFD:-LENFD, LENFD:-LENFD]
                    for q in range(9)])
    if hasattr(s, "close"):
        s.close()
    return out


def convergence_orders(sols):
    """Observed orders from solutions at levels 0..L: differences of successive levels
    taken on the level-0 nodes (every 2^l-th node of level l), relative to the finest
    solution's norm there; order_l = log2(e_l / e_{l+1})."""
    coarse = [u[:, ::2 ** l, ::2 ** l, ::2 ** l] for l, u in enumerate(sols)]
    ref = np.sqrt(np.sum(coarse[-1] ** 2))
    errs = [float(np.sqrt(np.sum((coarse[l] - coarse[l + 1]) ** 2)) / ref) for l in range(len(sols) - 1)]
    orders = [float(np.log2(errs[l] / errs[l + 1])) for l in range(len(errs) - 1)]
    return errs, orders


# ---- wave speeds ---------------------------------------------------------------------------
def _uniform_solver(make, n, th, ph, r, dr, dang, stept):
    """A solver on the uniform spherical grid of convergence_grid with the exact metric,
    the homogeneous medium (VP, VS, RHO), no PML, no free surface."""
    s = make(n, n, n, stept, False)
    s.set_coord(th.astype(np.float32), ph.astype(np.float32), r.astype(np.float32))
    nx = n + 2 * LENFD
    s.set_metric(np.sin(th).astype(np.float32), (1.0 / np.tan(th)).astype(np.float32),
                 np.full(nx, 1.0 / dang, np.float32), np.full(nx, 1.0 / dang, np.float32),
                 np.full(nx, 1.0 / dr, np.float32))
    shape = (nx, nx, nx)
    mu = RHO * VS * VS
    lam = RHO * VP * VP - 2 * mu
    s.set_media(np.full(shape, lam, np.float32, order="F"), np.full(shape, mu, np.float32, order="F"),
                np.full(shape, RHO, np.float32, order="F"))
    s.set_pml(np.zeros(6, np.int32), np.zeros(6, np.float32), np.ones(6, np.float32), np.zeros(6, np.float32))
    return s


def pulse_line(make, kind, level=1, width_km=3.0, t_end=2.4):
    """A pure P or pure S pulse in the homogeneous cube of convergence_grid (48 km, spacing
    1 km / 2^level, CFL 0.3 steps to t_end) against the closed-form solution of the wave
    equation at VP or VS, on the theta line through the centre (a > 0).

    P: an isotropic stress pulse sigma_ii = g = 1e6 exp(-d^2/w^2) Pa at rest.  The motion
    stays irrotational, v = grad(psi) with rho psi_tt = (lambda + 2 mu) lap(psi), psi(0) = 0,
    psi_t(0) = g / rho, so psi = 1e6 w^2 / (4 r VP rho) (exp(-(r - VP t)^2/w^2) -
    exp(-(r + VP t)^2/w^2)) and the radial velocity (v_theta on the line) is dpsi/dr.
    S: a rotational velocity pulse v = (dq/db, -dq/da, 0), q = exp(-d^2/w^2) (a, b the
    distances along theta and phi), at zero stress.  The motion stays divergence-free, each
    velocity component obeys the scalar wave equation at VS with zero initial rate, so
    v_phi = -dQ/da with Q = ((r - VS t) q(r - VS t) + (r + VS t) q(r + VS t)) / (2 r), and on
    the line d/da = d/dr.
    Returns (distances, numerical, closed-form) float64 arrays along the line."""
    n, th, ph, r, dr, dang = convergence_grid(level)
    stept = 0.3 * dr / VP
    c = LENFD + (n - 1) // 2
    # Cartesian offsets from the centre node in its local frame (theta, phi, r unit vectors)
    T, P_, Rr = np.meshgrid(th, ph, r, indexing="ij")
    X = np.stack([Rr * np.sin(T) * np.cos(P_), Rr * np.sin(T) * np.sin(P_), Rr * np.cos(T)])
    t0, p0 = th[c], ph[c]
    et = np.array([np.cos(t0) * np.cos(p0), np.cos(t0) * np.sin(p0), -np.sin(t0)])
    ep = np.array([-np.sin(p0), np.cos(p0), 0.0])
    er = np.array([np.sin(t0) * np.cos(p0), np.sin(t0) * np.sin(p0), np.cos(t0)])
    D = X - X[:, c, c, c][:, None, None, None]
    A = np.tensordot(et, D, axes=1)
    B = np.tensordot(ep, D, axes=1)
    H = np.tensordot(er, D, axes=1)
    w = width_km * 1000.0
    g = np.exp(-(A * A + B * B + H * H) / (w * w))
    s = _uniform_solver(make, n, th, ph, r, dr, dang, stept)
    if kind == "P":
        p = np.asfortranarray((1.0e6 * g).astype(np.float32))
        for comp in ("Txx", "Tyy", "Tzz"):
            s.set_field(comp, p)
        comp = 0
    else:
        s.set_field("Vx", np.asfortranarray((-2.0 * B / (w * w) * g).astype(np.float32)))
        s.set_field("Vy", np.asfortranarray((2.0 * A / (w * w) * g).astype(np.float32)))
        comp = 1
    steps = int(round(t_end / stept))
    s.run(steps)
    t = steps * stept
    line = slice(c + 1, LENFD + n)
    num = np.asarray(s.get_field(comp), np.float64)[line, c, c]
    if hasattr(s, "close"):
        s.close()
    d = np.sqrt(A[line, c, c] ** 2 + B[line, c, c] ** 2 + H[line, c, c] ** 2)
    if kind == "P":
        def psi(x):
            return 1.0e6 * w * w / (4.0 * x * VP * RHO) * (np.exp(-((x - VP * t) / w) ** 2) -
                                                             np.exp(-((x + VP * t) / w) ** 2))
        f = psi
    else:
        def f(x):
            q = lambda y: np.exp(-(y / w) ** 2)  # noqa: E731
            return -((x - VS * t) * q(x - VS * t) + (x + VS * t) * q(x + VS * t)) / (2.0 * x)
    e = 1.0e-3 * dr
    exact = (f(d + e) - f(d - e)) / (2.0 * e)
    return d, num, exact


# ---- Rayleigh waves on the free surface ----------------------------------------------------
def rayleigh_ratio(kappa):
    """c_R / Vs of a homogeneous half-space with Vp / Vs = kappa: the root in (0.5, 1) of
    (2 - x^2)^2 = 4 sqrt(1 - x^2) sqrt(1 - x^2 / kappa^2), by bisection."""
    f = lambda x: (2 - x * x) ** 2 - 4 * np.sqrt(1 - x * x) * np.sqrt(1 - x * x / (kappa * kappa))  # noqa: E731
    lo, hi = 0.5, 0.99
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if f(lo) * f(mid) <= 0:
            hi = mid
        else:
            lo = mid
    return 0.5 * (lo + hi)


def rayleigh_speed(make, dh_km):
    """Speed of the Rayleigh pulse of a vertical surface force (0.5 Hz Ricker centred at
    2.5 s) on a homogeneous half-space (VP, VS, RHO), 70 x 24 x 20 km at spacing dh_km,
    CFS-PML of 5 km on five faces, free surface on top: vertical velocity at surface
    receivers 8, 10, ..., 26 km from the source along theta; the delay of each trace
    against the nearest one by cross-correlation (parabolic peak), and the speed from a
    least-squares line of distance against delay.  Returns (measured, theoretical c_R) in
    m/s."""
    n_h, n_j, n_k = int(round(70 / dh_km)), int(round(24 / dh_km)), int(round(20 / dh_km))
    m = inputs.make_model(n_h, n_j, n_k, seed=1, dh_km=dh_km, z_top_km=dh_km, z_bottom_km=dh_km,
                          npml=int(round(5 / dh_km)), nrecv=0, source="surface", fc=0.5, t0=2.5, cfl=0.3)
    mu = RHO * VS * VS
    m.lam[:] = RHO * VP * VP - 2 * mu
    m.mu[:] = mu
    m.rho[:] = RHO
    m.stept = float(np.float32(0.3 * dh_km * 1000.0 * np.sin(m.x[LENFD:-LENFD]).min() / VP))
    m.pml_velocity[:] = VP
    ic, jc, kc = (int(v) for v in m.force_indx[0])
    step = int(round(2 / dh_km))
    offs = np.arange(int(round(8 / dh_km)), int(round(26 / dh_km)) + 1, step)
    rec = np.array([[ic + o, jc, kc] for o in offs], np.int32)
    s = make(m.ni, m.nj, m.nk, m.stept, True)
    inputs.attach(s, m)
    s.set_receivers(rec, 1)
    s.run(int(13.0 / m.stept))
    vz = np.asarray(s.get_seismo()[2], np.float64)      # (samples, receivers)
    if hasattr(s, "close"):
        s.close()
    r_top = float(m.z[-1 - LENFD])
    d = (m.x[rec[:, 0] - 1].astype(np.float64) - float(m.x[ic - 1])) * r_top
    lag = []
    for q in range(len(offs)):
        cc = np.correlate(vz[:, q], vz[:, 0], "full")
        k = int(np.argmax(cc))
        y0, y1, y2 = cc[k - 1], cc[k], cc[k + 1]
        lag.append((k - (vz.shape[0] - 1) + 0.5 * (y0 - y2) / (y0 - 2.0 * y1 + y2)) * m.stept)
    return float(np.polyfit(np.array(lag), d, 1)[0]), rayleigh_ratio(VP / VS) * VS
