"""Seeded synthetic inputs in the reference's layouts.

The reference's preprocessors write per-rank NetCDF files that the solver reads
(coord, metric, media, source, station).  No input data ships with the reference, so
the workloads are generated here with the same arithmetic the preprocessors use where
it matters for the solver:

* coordinates: seis3d_grid.F90:89-149 (uniform step or explicit list, degrees to
  radians, ghosts extrapolated linearly), in FP32 like the reference;
* sources: seis3d_source.F90:75-117 (nearest node, fractional shift, surface
  sources pinned to k = nk2);
* receivers: seis3d_station.F90:64-105 (nearest node; surface receivers on k = nk2);
* media: values sampled at the nodes of a 1-D layered model (Vs = Vp/1.73, Gardner
  density) with an optional seeded Gaussian-correlated perturbation.  The effective
  medium averaging of seis3d_media is not applied (both the solver and the oracle read
  the same node values).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

LENFD = 3
R_EARTH_KM = 6371.0


@dataclass
class Model:
    ni: int
    nj: int
    nk: int
    stept: float
    x: np.ndarray   # (nx,) colatitude, rad
    y: np.ndarray   # (ny,) longitude, rad
    z: np.ndarray   # (nz,) radius, m
    lam: np.ndarray  # (nx, ny, nz) Fortran-ordered semantics (index [i,j,k])
    mu: np.ndarray
    rho: np.ndarray
    pml_number: np.ndarray = field(default_factory=lambda: np.zeros(6, np.int32))
    pml_velocity: np.ndarray = field(default_factory=lambda: np.zeros(6, np.float32))
    pml_bmax: np.ndarray = field(default_factory=lambda: np.ones(6, np.float32))
    pml_amax: np.ndarray = field(default_factory=lambda: np.zeros(6, np.float32))
    free_surface: bool = True
    # forces: 1-based Fortran indices (num,3), shifts (num,3), start times (num,),
    # windows stf_time/stf_freq (ntwin,), amplitudes (num, ntwin)
    force_indx: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    force_shift: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    force_t0: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    stf_time: np.ndarray = field(default_factory=lambda: np.zeros(1, np.float32))
    stf_freq: np.ndarray = field(default_factory=lambda: np.zeros(1, np.float32))
    fx: np.ndarray = field(default_factory=lambda: np.zeros((0, 1), np.float32))
    fy: np.ndarray = field(default_factory=lambda: np.zeros((0, 1), np.float32))
    fz: np.ndarray = field(default_factory=lambda: np.zeros((0, 1), np.float32))
    stf_id: int = 200
    recv_indx: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    recv_tinv: int = 1
    name: str = ""

    @property
    def shape(self):
        return (self.ni + 6, self.nj + 6, self.nk + 6)

    @property
    def npoints(self):
        return self.ni * self.nj * self.nk


def grid_coords(n: int, step: float | None, origin: float, values: np.ndarray | None, to_si: float,
                degrees: bool, top_anchored: bool = False) -> np.ndarray:
    """One axis of read_grid_coord (seis3d_grid.F90:89-149) for a single domain."""
    nx = n + 2 * LENFD
    g = np.zeros(nx, np.float32)
    i1 = LENFD  # 0-based index of the first interior point
    if values is None:
        idx = np.arange(nx)
        if top_anchored:  # gz(k) = (k - num_z + LenFD)*dh + rmax
            g[:] = ((idx - (nx - 1) + LENFD).astype(np.float32) * np.float32(step) + np.float32(origin))
        else:             # gx(i) = (i - ni1)*dh + x0
            g[:] = ((idx - i1).astype(np.float32) * np.float32(step) + np.float32(origin))
    else:
        v = np.asarray(values, np.float32)
        assert v.size == n
        g[i1:i1 + n] = v
    if degrees:
        g = (g.astype(np.float64) / 180.0 * np.pi).astype(np.float32)
    else:
        g = (g * np.float32(to_si)).astype(np.float32)
    i2 = i1 + n - 1
    for q in range(1, LENFD + 1):
        g[i1 - q] = np.float32(np.float32(g[i1 - q + 1] + g[i1]) - g[i1 + 1])
        g[i2 + q] = np.float32(np.float32(g[i2 + q - 1] + g[i2]) - g[i2 - 1])
    return g


def stretched_depths_km(nk: int, top_km: float = 0.5, bottom_km: float = 2.0) -> np.ndarray:
    """Radii list (km, bottom to top) with spacing growing geometrically from top_km at
    the surface to bottom_km at the bottom (the `<z` list form of the grid input)."""
    if nk < 2:
        raise ValueError("nk >= 2")
    ratio = (bottom_km / top_km) ** (1.0 / max(nk - 2, 1))
    h = top_km * ratio ** np.arange(nk - 1)  # spacings from the top down
    depth = np.concatenate([[0.0], np.cumsum(h)])  # depth of node from the top
    r = R_EARTH_KM - depth[::-1]  # bottom to top
    return r.astype(np.float32)


def layered_media(x, y, z, seed: int, vp_top=5.8, vp_bottom=8.0, nlayers=4, perturb: float = 0.0,
                  corr_km: float = 10.0):
    """Node-sampled 1-D layered medium (Vp in km/s from vp_top to vp_bottom across
    seeded interfaces), Vs = Vp/1.73, rho = 1.741 Vp^0.25 g/cm^3, optional Gaussian-
    correlated relative perturbation of Vp and Vs scaled to max |dv| = perturb.
    Returns lam, mu, rho (SI) with shape (nx, ny, nz), Fortran-ordered."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = x.size, y.size, z.size
    ztop = float(z[nz - 1 - LENFD])
    depth_km = (ztop - z.astype(np.float64)) / 1000.0
    dmax = max(float(depth_km[LENFD]), 1e-3)
    iface = np.sort(rng.uniform(0.05, 0.9, nlayers - 1)) * dmax
    vps = np.linspace(vp_top, vp_bottom, nlayers)
    layer = np.searchsorted(iface, depth_km, side="right")
    vp1 = vps[np.clip(layer, 0, nlayers - 1)]  # (nz,)
    vp = np.broadcast_to(vp1[None, None, :], (nx, ny, nz)).astype(np.float64).copy()
    vs = vp / 1.73
    if perturb > 0.0:
        dv = gaussian_field((nx, ny, nz), x, y, z, corr_km, rng)
        dv *= perturb / max(np.abs(dv).max(), 1e-30)
        vp *= 1.0 + dv
        vs *= 1.0 + dv
    rho = 1.741 * vp ** 0.25 * 1000.0          # kg/m^3
    vp_ms, vs_ms = vp * 1000.0, vs * 1000.0
    mu = rho * vs_ms ** 2
    lam = rho * vp_ms ** 2 - 2.0 * mu
    # stored in Fortran order (first index fastest), the layout of the reference's arrays
    # and of the C ABI, so handing them to a solver needs no transposition
    return tuple(np.asfortranarray(a, dtype=np.float32) for a in (lam, mu, rho))


def gaussian_field(shape, x, y, z, corr_km, rng):
    """Zero-mean Gaussian random field with a Gaussian correlation of length corr_km,
    filtered in the Fourier domain on the (roughly uniform) node spacing."""
    nx, ny, nz = shape
    r_top = float(z[-1 - LENFD])
    dx = abs(float(x[LENFD + 1] - x[LENFD])) * r_top / 1000.0
    dy = abs(float(y[LENFD + 1] - y[LENFD])) * r_top / 1000.0 * np.sin(float(x[nx // 2]))
    dz = abs(float(np.mean(np.diff(z[LENFD:-LENFD])))) / 1000.0
    noise = rng.standard_normal(shape)
    kx = np.fft.fftfreq(nx, d=dx)[:, None, None]
    ky = np.fft.fftfreq(ny, d=dy)[None, :, None]
    kz = np.fft.rfftfreq(nz, d=dz)[None, None, :]
    filt = np.exp(-(np.pi * corr_km) ** 2 * (kx ** 2 + ky ** 2 + kz ** 2) / 2.0)
    f = np.fft.irfftn(np.fft.rfftn(noise) * filt, s=shape, axes=(0, 1, 2))
    f -= f.mean()
    return f / max(f.std(), 1e-30)


def locate(coord: np.ndarray, v: float) -> int:
    """minloc(abs(coord - v)) as a 1-based index (first minimum wins, like Fortran)."""
    return int(np.argmin(np.abs(coord - np.float32(v)))) + 1


def source_shift(coord: np.ndarray, i: int, v: float) -> float:
    """Fractional offset of a source from its node (seis3d_source.F90:100-116)."""
    c = coord
    i0 = i - 1
    if v > c[i0]:
        return float(np.float32((np.float32(v) - c[i0]) / (c[i0 + 1] - c[i0])))
    return float(np.float32((np.float32(v) - c[i0]) / (c[i0] - c[i0 - 1])))


def make_model(ni, nj, nk, seed=0, dh_km=1.0, theta_c_deg=50.0, phi_c_deg=100.0, z_top_km=0.5,
               z_bottom_km=2.0, npml=12, free_surface=True, nrecv=16, cfl=0.5, perturb=0.0,
               source="surface", force=(0.0, 0.0, 1.0e15), fc=0.2, t0=7.5, name="") -> Model:
    """A seeded model of the benchmark workloads (C1-C5): 1 km horizontal spacing (in degrees at
    the top radius), vertical spacing stretched from z_top_km to z_bottom_km, layered
    medium, CFS-PML of npml cells on x1 x2 y1 y2 z1 (+z2 without a free surface), one
    Ricker point force and nrecv seeded surface receivers."""
    rng = np.random.default_rng(seed + 7919)
    dh_deg = dh_km / R_EARTH_KM * 180.0 / np.pi
    theta0 = theta_c_deg - dh_deg * (ni - 1) / 2.0
    phi0 = phi_c_deg - dh_deg * (nj - 1) / 2.0
    x = grid_coords(ni, dh_deg, theta0, None, 1.0, degrees=True)
    y = grid_coords(nj, dh_deg, phi0, None, 1.0, degrees=True)
    zl = stretched_depths_km(nk, z_top_km, z_bottom_km)
    z = grid_coords(nk, None, 0.0, zl, 1000.0, degrees=False)
    lam, mu, rho = layered_media(x, y, z, seed, perturb=perturb)
    vpmax = float(np.sqrt((lam + 2 * mu) / rho)[LENFD:-LENFD, LENFD:-LENFD, LENFD:-LENFD].max())
    r_top = float(z[-1 - LENFD])
    hmin = min(float(np.min(np.diff(z[LENFD:-LENFD]))), dh_km * 1000.0 * float(np.sin(x[LENFD:-LENFD]).min()),
               dh_km * 1000.0)
    stept = cfl * hmin / vpmax
    m = Model(ni, nj, nk, float(np.float32(stept)), x, y, z, lam, mu, rho, name=name)
    m.free_surface = free_surface
    faces = [npml, npml, npml, npml, npml, 0 if free_surface else npml]
    m.pml_number = np.array(faces, np.int32)
    m.pml_velocity = np.full(6, 8000.0, np.float32)
    m.pml_bmax = np.full(6, 2.0, np.float32)
    m.pml_amax = np.full(6, np.float32(np.pi * fc), np.float32)
    nx, ny, nz = ni + 6, nj + 6, nk + 6
    ic, jc = LENFD + ni // 2 + 1, LENFD + nj // 2 + 1  # 1-based centre node
    if source == "surface":
        kc = nk + LENFD  # nk2 (1-based)
        shift = (0.0, 0.0, 0.0)
    elif source == "buried":
        kc = nk + LENFD - max(6, nk // 4)
        # an off-node position to exercise the fractional shift
        xs = float(x[ic - 1]) + 0.3 * float(x[ic] - x[ic - 1])
        ys = float(y[jc - 1]) - 0.2 * float(y[jc - 1] - y[jc - 2])
        zs = float(z[kc - 1]) + 0.25 * float(z[kc] - z[kc - 1])
        ic, jc, kc = locate(x, xs), locate(y, ys), locate(z, zs)
        shift = (source_shift(x, ic, xs), source_shift(y, jc, ys), source_shift(z, kc, zs))
    else:
        raise ValueError(source)
    m.force_indx = np.array([[ic, jc, kc]], np.int32)
    m.force_shift = np.array([shift], np.float32)
    m.force_t0 = np.zeros(1, np.float32)
    m.stf_time = np.array([t0], np.float32)
    m.stf_freq = np.array([fc], np.float32)
    m.fx = np.array([[force[0]]], np.float32)
    m.fy = np.array([[force[1]]], np.float32)
    m.fz = np.array([[force[2]]], np.float32)
    m.stf_id = 200
    # receivers on the surface away from the PML
    lo_i, hi_i = LENFD + npml + 3, LENFD + ni - npml - 2
    lo_j, hi_j = LENFD + npml + 3, LENFD + nj - npml - 2
    if hi_i < lo_i:
        lo_i, hi_i = LENFD + 1, LENFD + ni
    if hi_j < lo_j:
        lo_j, hi_j = LENFD + 1, LENFD + nj
    ri = rng.integers(lo_i, hi_i + 1, nrecv)
    rj = rng.integers(lo_j, hi_j + 1, nrecv)
    rk = np.full(nrecv, nk + LENFD)
    m.recv_indx = np.stack([ri, rj, rk], axis=1).astype(np.int32)
    m.recv_tinv = 1
    return m


def gaussian_hill(m: Model, amplitude_m: float, width_km: float | None = None, seed: int = 0,
                  centre: tuple | None = None) -> np.ndarray:
    """Heights (nx, ny) float32, Fortran order, of a seeded Gaussian hill for the terrain-
    following grid: h = A exp(-d^2 / w^2), d the arc distance (at the top radius) from the
    centre.  Seeded: the centre within the middle fifth of the surface, the width w in
    [0.12, 0.18] of the smaller horizontal extent (unless given)."""
    rng = np.random.default_rng(seed + 2718)
    r_top = float(m.z[-1 - LENFD])
    th = m.x.astype(np.float64)
    ph = m.y.astype(np.float64)
    if centre is None:
        ci = LENFD + m.ni // 2 + int(rng.integers(-m.ni // 10, m.ni // 10 + 1))
        cj = LENFD + m.nj // 2 + int(rng.integers(-m.nj // 10, m.nj // 10 + 1))
    else:
        ci, cj = centre
    if width_km is None:
        ext = min(m.ni * (th[LENFD + 1] - th[LENFD]), m.nj * (ph[LENFD + 1] - ph[LENFD]) * np.sin(th[ci])) * r_top
        width_km = float(rng.uniform(0.12, 0.18)) * ext / 1000.0
    dth = (th - th[ci])[:, None] * r_top
    dph = (ph - ph[cj])[None, :] * r_top * np.sin(th[ci])
    d2 = (dth ** 2 + dph ** 2) / (width_km * 1000.0) ** 2
    return np.asfortranarray((amplitude_m * np.exp(-d2)).astype(np.float32))


def config_c1(seed=0, **kw) -> Model:
    """C1 workload: 100x100x60, 1 km horizontal, 0.5-2 km vertical, layered Vp 5.8-8.0,
    12-cell PML on 5 faces, free surface, vertical Ricker force (0.2 Hz) at the surface
    centre, 16 seeded surface receivers, CFL 0.5 (flat top)."""
    return make_model(100, 100, 60, seed=seed, name="C1 100x100x60", **kw)


def config_c2(seed=0, component=2, **kw) -> Model:
    """C2 workload: 400x400x200 with a +/-5% Gaussian-correlated (10 km) Vp/Vs perturbation,
    64 surface receivers; component selects the force direction (0 Fx, 1 Fy, 2 Fz)."""
    f = [0.0, 0.0, 0.0]
    f[component] = 1.0e15
    return make_model(400, 400, 200, seed=seed, nrecv=64, perturb=0.05, force=tuple(f),
                      name=f"C2 400x400x200 F{'xyz'[component]}", **kw)


C4_STATIONS = ((-40, 0), (40, 0))  # (di, dj) of stations A and B from the surface centre, 1 km cells


def config_c4(seed=0, station=0, **kw) -> Model:
    """C4 workload (precision study): 256x256x128 with the C2 physics (+/-5% perturbation),
    a vertical surface force at station A (station=0) or B (station=1), 80 km apart on the
    surface; receivers: A, B, then 16 seeded surface receivers.  The two simulations are
    the source-side and receiver-side strain Green's tensors of the station pair."""
    m = make_model(256, 256, 128, seed=seed, nrecv=16, perturb=0.05, name=f"C4 256x256x128 station {'AB'[station]}",
                   **kw)
    ic, jc = LENFD + m.ni // 2 + 1, LENFD + m.nj // 2 + 1
    kc = m.nk + LENFD
    st = [(ic + di, jc + dj, kc) for di, dj in C4_STATIONS]
    m.force_indx = np.array([st[station]], np.int32)
    m.recv_indx = np.concatenate([np.array(st, np.int32), m.recv_indx]).astype(np.int32)
    return m


def config_c3(seed=0, count=32, **kw) -> list:
    """C3 workload: `count` virtual sources of seeded uneven sizes (horizontal 160-320 cells,
    depth 80-160 cells), the C2 physics (+/-5% perturbation), one vertical surface force
    at a seeded station each, 16 surface receivers."""
    rng = np.random.default_rng(seed + 104729)
    out = []
    for n in range(count):
        ni, nj = (int(v) for v in rng.integers(160, 321, 2))
        nk = int(rng.integers(80, 161))
        m = make_model(ni, nj, nk, seed=seed * 1000 + n, nrecv=16, perturb=0.05,
                       name=f"C3 #{n} {ni}x{nj}x{nk}", **kw)
        di = int(rng.integers(-ni // 4, ni // 4 + 1))
        dj = int(rng.integers(-nj // 4, nj // 4 + 1))
        m.force_indx = np.array([[LENFD + ni // 2 + 1 + di, LENFD + nj // 2 + 1 + dj, nk + LENFD]], np.int32)
        out.append(m)
    return out


def attach(solver, m: Model, metric: dict | None = None):
    """Feed a Model to a Solver (or any object with the same set-up methods)."""
    solver.set_coord(m.x, m.y, m.z)
    if metric is None:
        solver.compute_metric()
    else:
        solver.set_metric(metric["xsin"], metric["xcot"], metric["xi_x"], metric["eta_y"], metric["zeta_z"])
    solver.set_media(m.lam, m.mu, m.rho)
    solver.set_pml(m.pml_number, m.pml_velocity, m.pml_bmax, m.pml_amax)
    if m.force_indx.shape[0] > 0:
        solver.set_forces(m.force_indx, m.force_shift, m.force_t0, m.stf_time, m.stf_freq, m.fx, m.fy, m.fz,
                          m.stf_id)
    if m.recv_indx.shape[0] > 0:
        solver.set_receivers(m.recv_indx, m.recv_tinv)
    return solver


# ---- the reference's input files -----------------------------------------------------------
SUFFIX = "mpi000000"


def write_inputs(m: Model, root: str, metric: dict | None = None):
    """Write a Model as the reference's one-rank input files (NetCDF classic, the schemas
    of seis3d_grid/metric/media/source/station): coord_, metric_, media_, source_ and
    station_mpi000000.nc in `root`.  The metric defaults to the FP64 formula rounded to
    FP32 (seis3d_metric.F90:83-112 computed in double)."""
    import os

    from scipy.io import netcdf_file
    os.makedirs(root, exist_ok=True)
    f32 = np.float32

    def grid_file(name, arrays):
        with netcdf_file(os.path.join(root, f"{name}_{SUFFIX}.nc"), "w", version=1) as f:
            f.createDimension("I", m.x.size)
            f.createDimension("J", m.y.size)
            f.createDimension("K", m.z.size)
            for var, dim, a in arrays:
                v = f.createVariable(var, "f4", (dim,))
                v[:] = np.asarray(a, f32)

    grid_file("coord", [("x", "I", m.x), ("y", "J", m.y), ("z", "K", m.z)])
    if metric is None:
        metric = metric_fp64(m.x, m.y, m.z)
    grid_file("metric", [("xsin", "I", metric["xsin"]), ("xcot", "I", metric["xcot"]), ("xi_x", "I", metric["xi_x"]),
                         ("eta_y", "J", metric["eta_y"]), ("zeta_z", "K", metric["zeta_z"])])
    with netcdf_file(os.path.join(root, f"media_{SUFFIX}.nc"), "w", version=1) as f:
        f.createDimension("I", m.x.size)
        f.createDimension("J", m.y.size)
        f.createDimension("K", m.z.size)
        for var, a in (("lambda", m.lam), ("mu", m.mu), ("rho", m.rho)):
            v = f.createVariable(var, "f4", ("K", "J", "I"))
            v[:] = np.asarray(a, f32).transpose(2, 1, 0)
    nf = int(m.force_indx.shape[0])
    with netcdf_file(os.path.join(root, f"source_{SUFFIX}.nc"), "w", version=1) as f:
        f.createDimension("geo_dimension", 3)
        f.number_of_force = np.int32(nf)
        f.number_of_moment = np.int32(0)
        if nf > 0:
            ntw = int(np.asarray(m.stf_time).size)
            f.createDimension("force_point", nf)
            f.createDimension("force_time_window", ntw)
            for var, a in (("Fx", m.fx), ("Fy", m.fy), ("Fz", m.fz)):  # Fortran (ntwin, num)
                v = f.createVariable(var, "f4", ("force_point", "force_time_window"))
                v[:] = np.asarray(a, f32).reshape(nf, ntw)
            v = f.createVariable("force_indx", "i4", ("force_point", "geo_dimension"))
            v[:] = np.asarray(m.force_indx, np.int32)
            v = f.createVariable("force_axis", "f4", ("force_point", "geo_dimension"))
            v[:] = np.zeros((nf, 3), f32)
            v = f.createVariable("force_shift", "f4", ("force_point", "geo_dimension"))
            v[:] = np.asarray(m.force_shift, f32)
            v = f.createVariable("force_start_time", "f4", ("force_point",))
            v[:] = np.asarray(m.force_t0, f32)
            v = f.createVariable("force_stf_time", "f4", ("force_time_window",))
            v[:] = np.asarray(m.stf_time, f32)
            v = f.createVariable("force_stf_freq", "f4", ("force_time_window",))
            v[:] = np.asarray(m.stf_freq, f32)
            f.force_stf_id = np.int32(m.stf_id)
            f.force_stf_type = b"ricker" if m.stf_id == 200 else b"stf"
    npt = int(m.recv_indx.shape[0])
    with netcdf_file(os.path.join(root, f"station_{SUFFIX}.nc"), "w", version=1) as f:
        f.createDimension("num_pt", None)
        f.createDimension("geo_dim", 3)
        f.createDimension("twoelem", 2)
        for var, typ, a in (("indx", "i4", m.recv_indx), ("gindx", "i4", m.recv_indx),
                            ("coord", "f4", np.zeros((npt, 3))), ("grid", "f4", m.recv_indx)):
            v = f.createVariable(var, typ, ("num_pt", "geo_dim"))
            v[:npt] = np.asarray(a).astype(typ)
        v = f.createVariable("id", "i4", ("num_pt", "twoelem"))
        v[:npt] = np.stack([np.arange(1, npt + 1), np.ones(npt, int)], axis=1).astype(np.int32)
        f.tinv = np.int32(m.recv_tinv)
        f.title = b"station"


def metric_fp64(x, y, z):
    """seis3d_metric (seis3d_metric.F90:83-112) evaluated in double from the FP32
    coordinates and rounded to FP32: sin/cot of theta and the inverse of the mean of the
    forward and backward MacCormack derivatives of each coordinate (edges copied into the
    ghosts)."""
    coe_f = np.array([-0.30874, -0.6326, 1.2330, -0.3334, 0.04168])
    coe_b = np.array([-0.04168, 0.3334, -1.2330, 0.6326, 0.30874])

    def one(g):
        g = np.asarray(g, np.float32).astype(np.float64)
        n = g.size
        out = np.zeros(n)
        for i in range(n):
            ii = min(max(i, LENFD), n - 1 - LENFD)
            sb = sum(g[ii - 3 + q] * coe_b[q] for q in range(5))
            sf = sum(g[ii - 1 + q] * coe_f[q] for q in range(5))
            out[i] = 1.0 / ((sb + sf) * 0.5)
        return out.astype(np.float32)

    xs = np.asarray(x, np.float32).astype(np.float64)
    return {"xsin": np.sin(xs).astype(np.float32), "xcot": (1.0 / np.tan(xs)).astype(np.float32),
            "xi_x": one(x), "eta_y": one(y), "zeta_z": one(z)}


def write_conf(path: str, m: Model, nt: int, roots: dict, snaps=(), checkpoint_tinv=0, run_from_checkpoint=0):
    """A SeisFD3D.conf for `m` with the keys the solver reads (para_init, io_init,
    abs_init, io_snap_read).  roots: GRID_ROOT MEDIA_ROOT SOURCE_ROOT STATION_ROOT
    OUTPUT_ROOT CHECKPOINT_ROOT.  snaps: (subs, subc, subt, tinv, tcnt, "V"|"T"|"TV") with
    the reference's interior-relative indices (-1: first point / to the end, -2: surface)."""
    n = [int(v) for v in m.pml_number]
    lines = [f"ni = {m.ni}", f"nj = {m.nj}", f"nk = {m.nk}", f"nt = {int(nt)}", f"stept = {float(m.stept)!r}",
             "dims = 1 1 1", "# PML: x1 x2 y1 y2 z1 z2",
             "abs_number = " + " ".join(str(v) for v in n),
             "abs_velocity = " + " ".join(repr(float(v)) for v in m.pml_velocity),
             "CFS_bmax = " + " ".join(repr(float(v)) for v in m.pml_bmax),
             "CFS_amax = " + " ".join(repr(float(v)) for v in m.pml_amax)]
    for k in ("GRID_ROOT", "MEDIA_ROOT", "SOURCE_ROOT", "STATION_ROOT", "OUTPUT_ROOT", "CHECKPOINT_ROOT"):
        if k in roots:
            lines.append(f"{k} = {roots[k]}")
    lines += [f"checkpoint_tinv = {int(checkpoint_tinv)}", f"run_from_checkpoint = {int(run_from_checkpoint)}",
              f"number_of_snap = {len(snaps)}"]
    for q, (subs, subc, subt, tinv, tcnt, var) in enumerate(snaps, start=1):
        cols = " ".join(str(int(v)) for v in (*subs, *subc, *subt, tinv, tcnt))
        lines.append(f"snap_{q:03d} = {cols} {var}   # subs subc subt tinv tcnt")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


# ---- inputs of the sensitivity-kernel program (SI_ker_sta) ---------------------------------

def _f32text(v) -> str:
    """The shortest text that reads back as the same float32 value."""
    return repr(float(np.float32(v)))


def write_tomo_conf(path: str, main_conf: str, snap_id: int, roots: dict, knt: int, sgt_m0: float,
                    sub_start=(1, 1, 1), sub_count=(-1, -1, -1), sub_stride=(1, 1, 1), block_from=(1, 1, 1),
                    block_size=(-1, -1, -1), first_run=True, max_pick=4, filter_files=()):
    """TomoKernel.conf with the keys init_kernel and init_filter read
    (code/srcF.kernel/SI_ker_sta.F90:1047-1112).  roots: SGT_ROOT SGT_STAX SGT_STAY SGT_STAZ
    EVENT_ROOT EVENT_OUTD.  filter_files: one file name (or "none") per frequency band."""
    def row(key, vals):
        return f"{key} = " + " ".join(str(int(v)) for v in vals)
    lines = [f"MAIN_CONF = {main_conf}", f"snap_id = {int(snap_id)}",
             f"first_run = {'.true.' if first_run else '.false.'}",
             row("sub_start", sub_start), row("sub_count", sub_count), row("sub_stride", sub_stride),
             row("block_from", block_from), row("block_size", block_size),
             f"SGT_TIMEDIM_SIZE = {int(knt)}", f"SGT_M0 = {_f32text(sgt_m0)}"]
    for k in ("SGT_ROOT", "SGT_STAX", "SGT_STAY", "SGT_STAZ", "EVENT_ROOT", "EVENT_OUTD"):
        lines.append(f"{k} = {roots[k]}")
    lines += [f"maximum_of_pick_per_component = {int(max_pick)}", f"number_of_freqband = {len(filter_files)}",
              "<filter_file>"] + [str(f) for f in filter_files]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_filter_file(path: str, b, a):
    """A filter file: NOD1, then NOD1 lines of a and b in F20.16 (init_filter).  Returns the
    (b, a) coefficients as they read back."""
    b = np.asarray(b, np.float64)
    a = np.asarray(a, np.float64)
    rows = [f"{x:20.16f}{y:20.16f}" for x, y in zip(a, b)]
    if any(len(r) != 40 for r in rows):
        raise ValueError("coefficient does not fit F20.16")
    with open(path, "w") as f:
        f.write(f"{b.size}\n" + "\n".join(rows) + "\n")
    return np.array([float(r[20:]) for r in rows]), np.array([float(r[:20]) for r in rows])


def write_synthetic(path: str, t, v, u):
    """A synthetic file: one line of T V U per sample (init_synthetic)."""
    with open(path, "w") as f:
        for row in zip(t, v, u):
            f.write(" ".join(_f32text(x) for x in row) + "\n")


def write_event_list(path: str, events):
    """An event list: per event the header line (name, six pick counts, rot_mat column by
    column), three synthetic file names and the pick lines of components 1..6 (band,
    P1 | P2 | N, t1, t2, output directory).  events: dicts with name, picks (six lists of
    (band, filt, t1, t2, dir)), rot (3x3, rot[d, c]) and syn (three file names)."""
    lines = []
    for e in events:
        picks = e["picks"]
        rot = np.asarray(e["rot"], np.float32).reshape(3, 3)
        head = [e["name"]] + [str(len(p)) for p in picks] + [_f32text(x) for x in rot.flatten(order="F")]
        lines.append(" ".join(head))
        lines += list(e["syn"])
        for comp in picks:
            for band, filt, t1, t2, d in comp:
                lines.append(f"{int(band)} {filt} {_f32text(t1)} {_f32text(t2)} {d}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


# ---- inputs of the inversion (inv.LSQR solver_damp_smooth) ---------------------------------

def write_kernel_row_file(path: str, nblk: int, idx, coef, ker0: float = 1.0):
    """One measurement's kernel row for one component as the inversion reads it: Fortran
    unformatted sequential records (4-byte length markers) of (num_blk, ker0), (ncoef) and
    the ncoef pairs (1-based block index, single-precision coefficient)."""
    import struct
    idx = np.asarray(idx, np.int32)
    coef = np.asarray(coef, np.float32)
    pairs = np.empty(idx.size, dtype=[("i", "<i4"), ("c", "<f4")])
    pairs["i"], pairs["c"] = idx, coef

    def rec(payload: bytes) -> bytes:
        return struct.pack("<i", len(payload)) + payload + struct.pack("<i", len(payload))
    with open(path, "wb") as f:
        f.write(rec(struct.pack("<if", int(nblk), float(ker0))))
        f.write(rec(struct.pack("<i", idx.size)))
        f.write(rec(pairs.tobytes()))


def write_smoothing_file(path: str, nblk: int, rows):
    """The smoothing operator: num_blk, number of rows, widest row, total entries; then per
    row ncoef, its 1-based block indices and its coefficients.  rows: (idx, coef) pairs."""
    nel = sum(len(r[0]) for r in rows)
    nbd = max((len(r[0]) for r in rows), default=0)
    lines = [f"{int(nblk)} {len(rows)} {nbd} {nel}"]
    for idx, coef in rows:
        lines.append(" ".join([str(len(idx))] + [str(int(i)) for i in idx] + [_f32text(c) for c in coef]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


# ---- inputs of the medium preprocessor (seis3d_media) ---------------------------------------

def write_media_conf(path: str, background, perturbed=None, half_sample=(1, 1, 1)):
    """The media configuration init_media reads (code/srcF/seis3d_media.F90:264-338):
    background = (type, format, file name); perturbed likewise or None."""
    lines = ["half_sample_point = " + " ".join(str(int(v)) for v in half_sample),
             f"background_type = {background[0]}", f"background_format = {background[1]}",
             f"background_filename = {background[2]}"]
    if perturbed is None:
        lines.append("perturbed_type = none")
    else:
        lines += [f"perturbed_type = {perturbed[0]}", f"perturbed_format = {perturbed[1]}",
                  f"perturbed_filename = {perturbed[2]}"]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _units_lines(units):
    return [f"distance2meter = {units[0]!r}", f"velocity2m/s = {units[1]!r}", f"density2kg/m^3 = {units[2]!r}"]


def write_cart1d_file(path: str, z, rho, vp, vs, meaning="depth", units=(1.0, 1.0, 1.0)):
    """An ascii cart1d model (layer1d_read :341-430): one record z rho Vp Vs per sample;
    `meaning` axis, depth or thickness; units (distance, velocity, density) to SI."""
    lines = [f"radial_sampling = {len(z)}"] + _units_lines(units) + [f"radial_meaning = {meaning}", "<anchor_data>"]
    lines += [" ".join(_f32text(v) for v in row) for row in zip(z, rho, vp, vs)]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_layer_file(path: str, kind: str, x_deg, y_deg, v, vp, vs, rho, meaning="depth", units=(1.0, 1.0, 1.0)):
    """An ascii interface (kind "interface", v = interface heights (ni, nj, nk)) or layered
    (kind "layered", v = depths or thicknesses per `meaning`) model (interface_read :433-532,
    layered_read :535-643); vp, vs, rho (2, nk); x, y in degrees."""
    v = np.asarray(v, np.float32)
    ni, nj, nk = v.shape
    key = "number_of_interface" if kind == "interface" else "number_of_layer"
    lines = [f"{key} = {nk}"] + _units_lines(units) + [f"horizontal_sampling = {ni} {nj}"]
    if kind != "interface":
        lines.append(f"layer_meaning = {meaning}")
    lines.append("<anchor_media>")
    vp, vs, rho = (np.asarray(a, np.float32).reshape(2, nk, order="F") for a in (vp, vs, rho))
    for k in range(nk):
        lines.append(" ".join(_f32text(a[s, k]) for a in (vp, vs, rho) for s in range(2)))
    lines.append("<anchor_interface>" if kind == "interface" else "<anchor_layer>")
    for j in range(nj):
        for i in range(ni):
            lines.append(" ".join([_f32text(x_deg[i]), _f32text(y_deg[j])] + [_f32text(v[i, j, k]) for k in range(nk)]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _nc_fortran(f, name, a, dims):
    """a variable whose Fortran shape is a.shape, dimensions listed fastest first"""
    a = np.asarray(a, np.float32)
    v = f.createVariable(name, "f4", tuple(reversed(dims)))
    v[:] = a.transpose(tuple(reversed(range(a.ndim))))


def write_composite_nc(path: str, x_deg, y_deg, h, vp, vs, rho, vp_exp, vs_exp, rho_exp):
    """A composite model (composite_read :646-702): thickness (ni, nj, nk), Vp, Vs, rho
    (2, ni, nj, nk) and the exponents (nk)."""
    from scipy.io import netcdf_file
    h = np.asarray(h, np.float32)
    ni, nj, nk = h.shape
    with netcdf_file(path, "w", version=1) as f:
        for d, n in (("theta", ni), ("phi", nj), ("layer", nk), ("side", 2)):
            f.createDimension(d, n)
        _nc_fortran(f, "theta", x_deg, ("theta",))
        _nc_fortran(f, "phi", y_deg, ("phi",))
        _nc_fortran(f, "thickness", h, ("theta", "phi", "layer"))
        for name, a in (("Vp", vp), ("Vs", vs), ("rho", rho)):
            _nc_fortran(f, name, a, ("side", "theta", "phi", "layer"))
        for name, a in (("Vp_poly_d", vp_exp), ("Vs_poly_d", vs_exp), ("rho_poly_d", rho_exp)):
            _nc_fortran(f, name, a, ("layer",))


def write_volume_nc(path: str, x_deg, y_deg, rz, sealevel, vp, vs, rho):
    """A volume model (volume_init / volume_read :705-779): depth2sealevel (nk), global
    attribute sealevel, Vp, Vs, rho (ni, nj, nk)."""
    from scipy.io import netcdf_file
    vp = np.asarray(vp, np.float32)
    ni, nj, nk = vp.shape
    with netcdf_file(path, "w", version=1) as f:
        for d, n in (("theta", ni), ("phi", nj), ("depth", nk)):
            f.createDimension(d, n)
        f.sealevel = np.float32(sealevel)
        _nc_fortran(f, "theta", x_deg, ("theta",))
        _nc_fortran(f, "phi", y_deg, ("phi",))
        _nc_fortran(f, "depth2sealevel", rz, ("depth",))
        for name, a in (("Vp", vp), ("Vs", vs), ("rho", rho)):
            _nc_fortran(f, name, a, ("theta", "phi", "depth"))


def write_verpoly_nc(path: str, x_deg, y_deg, rz, sealevel, vp_c, vs_c, rho_c, vp_exp, vs_exp, rho_exp):
    """A verpoly model (verpoly_init / verpoly_read :782-850): depth2sealevel (ni, nj, nk),
    coefficients (ni, nj, nk, npoly), exponents (npoly), global attribute sealevel."""
    from scipy.io import netcdf_file
    vp_c = np.asarray(vp_c, np.float32)
    ni, nj, nk, npoly = vp_c.shape
    with netcdf_file(path, "w", version=1) as f:
        for d, n in (("theta", ni), ("phi", nj), ("depth", nk), ("polynomial", npoly)):
            f.createDimension(d, n)
        f.sealevel = np.float32(sealevel)
        _nc_fortran(f, "theta", x_deg, ("theta",))
        _nc_fortran(f, "phi", y_deg, ("phi",))
        _nc_fortran(f, "depth2sealevel", rz, ("theta", "phi", "depth"))
        for name, a in (("Vp_poly_c", vp_c), ("Vs_poly_c", vs_c), ("rho_poly_c", rho_c)):
            _nc_fortran(f, name, a, ("theta", "phi", "depth", "polynomial"))
        for name, a in (("Vp_poly_d", vp_exp), ("Vs_poly_d", vs_exp), ("rho_poly_d", rho_exp)):
            _nc_fortran(f, name, a, ("polynomial",))


def grid_c2(ni=400, nj=400, nk=200, dh_km=1.0, theta_c_deg=50.0, phi_c_deg=100.0, z_top_km=0.5, z_bottom_km=2.0):
    """The grid (x, y, z with ghosts; radians and metres) of make_model for a size."""
    dh_deg = dh_km / R_EARTH_KM * 180.0 / np.pi
    x = grid_coords(ni, dh_deg, theta_c_deg - dh_deg * (ni - 1) / 2.0, None, 1.0, degrees=True)
    y = grid_coords(nj, dh_deg, phi_c_deg - dh_deg * (nj - 1) / 2.0, None, 1.0, degrees=True)
    z = grid_coords(nk, None, 0.0, stretched_depths_km(nk, z_top_km, z_bottom_km), 1000.0, degrees=False)
    return x, y, z


def media_models(x, y, z, seed=0, nlayers=4, vp_top=5.8, vp_bottom=8.0, perturb=0.05, corr_km=10.0,
                 spacing_km=2.0):
    """Seeded inputs of the medium preprocessor for a grid: a cart1d background of nlayers
    constant-velocity layers (Vp from vp_top to vp_bottom km/s at seeded depths, each
    interface a repeated depth; Vs = Vp / 1.73, Gardner density) and, for perturb > 0, a
    volume perturbation of Vp and Vs (the same relative field, max |dv| = perturb, Gaussian
    correlation corr_km) sampled every spacing_km over the grid.  Returns the set-up calls
    of fwant_gb300.Media: [("set_cart1d", ...), ("set_volume", ...)]."""
    rng = np.random.default_rng(seed)
    f32 = np.float32
    ztop = float(z[-1 - LENFD])
    dmax = (ztop - float(z[0])) / 1000.0
    iface = np.sort(rng.uniform(0.05, 0.9, nlayers - 1)) * dmax
    vps = np.linspace(vp_top, vp_bottom, nlayers)
    d = [0.0]
    vp = [vps[0]]
    for q, dz in enumerate(iface):
        d += [dz, dz]
        vp += [vps[q], vps[q + 1]]
    d.append(dmax * 1.5)
    vp.append(vps[-1])
    d = (np.array(d) * 1000.0).astype(f32)
    vp = (np.array(vp) * 1000.0).astype(f32)
    calls = [("set_cart1d", (d, vp, (vp / f32(1.73)).astype(f32), (f32(1741.0) * (vp / f32(1000.0)) ** f32(0.25))))]
    if perturb > 0.0:
        r_km = ztop / 1000.0
        span_x = (float(x[-1]) - float(x[0])) * r_km
        span_y = (float(y[-1]) - float(y[0])) * r_km * np.sin(float(x[x.size // 2]))
        mi, mj = int(span_x / spacing_km) + 3, int(span_y / spacing_km) + 3
        mk = int(dmax * 1.2 / spacing_km) + 3
        mx = np.linspace(float(x[0]), float(x[-1]), mi).astype(f32)
        my = np.linspace(float(y[0]), float(y[-1]), mj).astype(f32)
        rz = np.linspace(-1000.0, dmax * 1200.0, mk).astype(f32)
        noise = rng.standard_normal((mi, mj, mk))
        k = [np.fft.fftfreq(n, d=spacing_km) for n in (mi, mj)] + [np.fft.rfftfreq(mk, d=spacing_km)]
        filt = np.exp(-(np.pi * corr_km) ** 2 * (k[0][:, None, None] ** 2 + k[1][None, :, None] ** 2
                                                 + k[2][None, None, :] ** 2) / 2.0)
        dv = np.fft.irfftn(np.fft.rfftn(noise) * filt, s=(mi, mj, mk), axes=(0, 1, 2))
        dv = (dv - dv.mean()) * perturb / max(np.abs(dv - dv.mean()).max(), 1e-30)
        dv = dv.astype(f32)
        calls.append(("set_volume", (1, mx, my, rz, f32(ztop), dv, dv.copy(), np.zeros_like(dv))))
    return calls
