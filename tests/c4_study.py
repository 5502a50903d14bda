"""C4 precision study: one station pair on a 256x256x128 grid.

Simulation A (vertical surface force at station A) is the source side and simulation B
(vertical force at station B) the receiver side of the pair's ZZ sensitivity kernel.
Both record the strain Green's tensor of a strided kernel block every TINV steps; the
kernel (SI_ker_sta.F90 sgt2scatter3 + scatter2kernel, component Z) uses the vertical
velocity V at station B from simulation A and its time integral U over a window that
holds the surface waves.

The FP64 reference is the double-precision CPU restatement with the metric kept in
double (tests/golden/make_c4_reference.py writes it to tests/golden/c4_fp64_reference.npz);
the GPU runs are repeated with FP32, BF16 and FP16 wavefield storage.
"""
import numpy as np

from fwant_gb300 import inputs

NT = 1000               # time steps of each simulation
TINV = 4                # SGT frame interval (steps)
KNT = NT // TINV        # frames per SGT series
SGT_M0 = 1.0e15
WINDOW_T1 = 12.0        # s: first frame of the kernel window
# kernel block (1-based indices with ghosts): laterally every 8th point away from the PML,
# vertically every 4th point from above the bottom PML to the surface
SUBS = (20, 20, 28)
SUBC = (28, 28, 26)
SUBT = (8, 8, 4)
NPTS = SUBC[0] * SUBC[1] * SUBC[2]


def models(seed=0):
    return [inputs.config_c4(seed=seed, station=s) for s in (0, 1)]


def block_media(m):
    idx = [np.arange(SUBS[d] - 1, SUBS[d] - 1 + SUBT[d] * SUBC[d], SUBT[d]) for d in range(3)]
    lam = m.lam[np.ix_(*idx)].transpose(2, 1, 0).reshape(-1)
    mu = m.mu[np.ix_(*idx)].transpose(2, 1, 0).reshape(-1)
    return np.ascontiguousarray(lam, np.float32), np.ascontiguousarray(mu, np.float32)


def window(stept):
    kdt = TINV * float(np.float32(stept))
    nt1 = int(np.ceil(WINDOW_T1 / kdt))
    return kdt, nt1, KNT


def kernel_waveforms(vz_b, stept):
    """V and U at the kernel frames from the full-rate vertical velocity at station B
    (sample s at ntime s+1): V(n) = v(ntime n*TINV); U is the trapezoid integral of v."""
    v = np.asarray(vz_b, np.float64)
    u = np.concatenate([[0.5 * v[0] * stept], 0.5 * stept * np.cumsum(v[:-1] + v[1:]) + 0.5 * v[0] * stept])
    sel = np.arange(1, KNT + 1) * TINV - 1
    return v[sel].astype(np.float32), u[sel].astype(np.float32)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
