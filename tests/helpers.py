"""Shared set-up for the parity tests: small seeded models fed identically to the
CUDA solver and to the oracle."""
import numpy as np

from fwant_gb300 import inputs

LENFD = 3


def small_model(kind="surface", ni=26, nj=22, nk=20, npml=4, seed=3):
    """Small variants covering every boundary path:
    surface  - free surface, force on the surface (SrcSurface traction path)
    buried   - free surface, off-node buried force (7^3 smoothing, surface renormalisation)
    nofree   - PML on all six faces, buried force (no free surface)
    moment   - free surface, buried moment-tensor source
    water    - like buried, with a fluid (mu = 0) layer below the source
    """
    if kind in ("surface",):
        m = inputs.make_model(ni, nj, nk, seed=seed, npml=npml, nrecv=6, source="surface", fc=2.0, t0=0.6)
    elif kind in ("buried", "moment", "water"):
        m = inputs.make_model(ni, nj, nk, seed=seed, npml=npml, nrecv=6, source="buried", fc=2.0, t0=0.6,
                              force=(3.0e14, -2.0e14, 1.0e15))
    elif kind == "nofree":
        m = inputs.make_model(ni, nj, nk, seed=seed, npml=npml, nrecv=6, source="buried", fc=2.0, t0=0.6,
                              free_surface=False, force=(1.0e15, 0.0, 5.0e14))
    else:
        raise ValueError(kind)
    if kind == "water":
        m.mu[:, :, LENFD + 2:LENFD + 5] = 0.0
        m.lam[:, :, LENFD + 2:LENFD + 5] = np.float32(2.2e9)
        m.rho[:, :, LENFD + 2:LENFD + 5] = np.float32(1000.0)
    # a second receiver set inside the volume exercises non-surface sampling
    extra = np.array([[LENFD + 5, LENFD + 6, LENFD + nk // 2], [LENFD + ni - 3, LENFD + 4, LENFD + 3]], np.int32)
    m.recv_indx = np.concatenate([m.recv_indx, extra])
    return m


MOMENT = dict(mom=np.array([1.0e15, -0.5e15, -0.5e15, 0.3e15, 0.2e15, -0.1e15], np.float32).reshape(6, 1, 1))


def feed(solver, m, metric, kind):
    inputs.attach(solver, m, metric=metric)
    if kind == "moment":
        solver.set_forces(np.zeros((0, 3), np.int32), np.zeros((0, 3)), np.zeros(0), m.stf_time, m.stf_freq,
                          np.zeros((0, 1)), np.zeros((0, 1)), np.zeros((0, 1)))
        solver.set_moments(m.force_indx, m.force_shift, m.force_t0, m.stf_time, m.stf_freq, MOMENT["mom"], 200)
    return solver


def interior(a):
    return a[LENFD:-LENFD, LENFD:-LENFD, LENFD:-LENFD]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.sqrt(np.sum(b * b))
    num = np.sqrt(np.sum((a - b) ** 2))
    return num / den if den > 0 else num
