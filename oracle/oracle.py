"""ORACLE — test infrastructure, never the product.

ctypes binding of the CPU restatements in fwant_oracle.cpp (the forward solver),
sgtker_oracle.cpp (the sensitivity-kernel accumulation), lsqr_oracle.cpp (the LSQR
inversion solver) and media_oracle.cpp (the medium preprocessor).  `Oracle` has the same
set-up methods as `fwant_gb300.Solver`, so a test feeds both from one Model.  Only the
tests, `__graft_entry__.smoke()` and the `cpu_baseline` leg of `bench.py` use it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "fwant_oracle.cpp"), os.path.join(HERE, "sgtker_oracle.cpp"),
        os.path.join(HERE, "lsqr_oracle.cpp"), os.path.join(HERE, "media_oracle.cpp")]
LIB = os.path.join(HERE, "_build", "libfwant_oracle.so")
COMPONENTS = ("Vx", "Vy", "Vz", "Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)
_vp = C.c_void_p
_SIGS = [
    ("orc_create", _vp, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int]),
    ("orc_destroy", None, [_vp]),
    ("orc_set_threads", C.c_int, [C.c_int]),
    ("orc_set_coord", None, [_vp, _dp, _dp, _dp]),
    ("orc_set_metric", None, [_vp, _dp, _dp, _dp, _dp, _dp]),
    ("orc_set_media", None, [_vp, _dp, _dp, _dp]),
    ("orc_set_pml", C.c_int, [_vp, _ip, _dp, _dp, _dp]),
    ("orc_set_srcsurface", None, [_vp, C.c_int]),
    ("orc_set_topography", None, [_vp, _dp]),
    ("orc_topography_array", None, [_vp, C.c_int, _dp]),
    ("orc_set_forces", None, [_vp, C.c_int, C.c_int, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int]),
    ("orc_set_moments", None, [_vp, C.c_int, C.c_int, _ip, _dp, _dp, _dp, _dp, _dp, C.c_int]),
    ("orc_set_receivers", None, [_vp, C.c_int, _ip, C.c_int]),
    ("orc_run", C.c_int, [_vp, C.c_int]),
    ("orc_ntime", C.c_int, [_vp]),
    ("orc_freenode", C.c_int, [_vp]),
    ("orc_get_field", None, [_vp, C.c_int, _dp]),
    ("orc_set_field", None, [_vp, C.c_int, _dp]),
    ("orc_get_pml_profile", None, [_vp, C.c_int, _dp, _dp, _dp]),
    ("orc_get_seismo", C.c_int, [_vp, _dp, C.c_int]),
    ("orc_last_error", C.c_char_p, [_vp]),
    ("orc_stf", C.c_double, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_int]),
    ("orc_norm_delt", C.c_int, [C.c_double, C.c_double, C.c_double, _dp]),
    ("orc_pml_R", C.c_double, [C.c_int]),
    ("orc_metric", None, [C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _fp]),
    ("orc_metric_dp", None, [C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _fp]),
    ("orc_op", C.c_double, [C.c_int, C.c_int, _dp, C.c_int]),
    ("orc_iir", None, [_dp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]),
    ("orc_metric_dd", None, [C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, _dp, _dp, _dp, _dp, _dp]),
    ("orc_stress2strain", None, [C.c_longlong, C.c_int, _fp, _fp, _fp, _fp]),
    ("orc_sgt2scatter3", None, [C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_double, _fp, _fp, _fp, _fp, _fp, _fp,
                                C.c_int, C.c_int, _dp]),
    ("orc_scatter2kernel", None, [C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_double, _fp, _fp, _dp, _dp,
                                  C.c_double, C.c_int, _dp, _dp, _dp, _dp]),
    ("orc_lsqr", C.c_longlong, [C.c_longlong, C.c_longlong, C.POINTER(C.c_longlong), _ip, _dp, _dp, C.c_double,
                                 C.c_double, C.c_longlong, _dp, _dp, _dp, _ip]),
    ("orc_lgtsol", None, [C.c_longlong, C.c_longlong, C.c_double, _dp, _dp]),
    ("orc_media_create", _vp, [C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, C.c_float, _ip]),
    ("orc_media_destroy", None, [_vp]),
    ("orc_media_last_error", C.c_char_p, [_vp]),
    ("orc_media_set_cart1d", None, [_vp, C.c_int, _fp, _fp, _fp, _fp]),
    ("orc_media_set_layers", None, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _fp,
                                    _fp, _fp]),
    ("orc_media_set_volume", None, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, C.c_float, _fp, _fp, _fp]),
    ("orc_media_set_verpoly", None, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, C.c_float, _fp,
                                     _fp, _fp, _fp, _fp, _fp]),
    ("orc_media_eval", C.c_int, [_vp, _fp, _fp, _fp]),
    ("orc_media_stept_check", None, [_vp, _fp, _fp, _fp, _fp, _ip, _fp, _fp]),
    ("orc_scatter2kernel_dv", None, [C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp, _dp,
                                     C.c_double, _dp, _dp, _dp, _dp]),
]


# The checker: every product and sum rounds separately (no FP contraction), as the
# reference's FP32 source expressions do, so the GPU's reference-order form can be compared
# bit for bit.
CHECK_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off"]
# The timed CPU baseline: the same sources built for speed (-O3 vectorisation and unrolling,
# fused multiply-adds allowed).  Results differ from the checker by rounding only; it is
# never used to check anything.  Generic target ISA (no -march=native), so one recipe
# builds on x86-64 and aarch64 hosts alike.
TIMING_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=fast", "-funroll-loops"]
TIMING_LIB = os.path.join(HERE, "_build", "libfwant_oracle_timing.so")


def _build_one(target, flags, force, verbose):
    os.makedirs(os.path.dirname(target), exist_ok=True)
    if not force and os.path.exists(target) and all(os.path.getmtime(target) >= os.path.getmtime(s) for s in SRCS):
        return target
    cmd = ["g++", *flags, "-o", target, *SRCS]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return target


def build(force: bool = False, verbose: bool = False, timing: bool = True) -> str:
    """Compile the oracle checker (g++, OpenMP, no FP contraction) and, unless timing is
    False, the timing-only build of the same sources."""
    if timing:
        _build_one(TIMING_LIB, TIMING_FLAGS, force, verbose)
    return _build_one(LIB, CHECK_FLAGS, force, verbose)


_LIBS = {}


def lib(timing: bool = False):
    """The checker library, or with timing=True the timing-only build (CPU baselines)."""
    path = TIMING_LIB if timing else LIB
    if path not in _LIBS:
        if not os.path.exists(path):
            _build_one(path, TIMING_FLAGS if timing else CHECK_FLAGS, False, False)
        L = C.CDLL(path)
        for name, res, args in _SIGS:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIBS[path] = L
    return _LIBS[path]


def build_flags(timing: bool = False) -> str:
    return " ".join(TIMING_FLAGS if timing else CHECK_FLAGS)


def _d(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def set_threads(n: int, timing: bool = False) -> int:
    return lib(timing).orc_set_threads(int(n))


def _f(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))


def stress2strain(lam, mu, stress):
    """stress: (6, knt, npts) Txx Tyy Tzz Txy Txz Tyz -> strains of the same shape (FP32)."""
    st = np.asarray(stress, np.float32)
    _, knt, npts = st.shape
    out = np.zeros(st.size, np.float32)
    lam_, mu_, s_ = _f(lam), _f(mu), _f(st)
    lib().orc_stress2strain(npts, knt, _p(lam_, C.c_float), _p(mu_, C.c_float), _p(s_, C.c_float),
                            _p(out, C.c_float))
    return out.reshape(st.shape)


def sgt2scatter3(lam, mu, rsgt, ssgt, dt, nt1=None, nt2=None, mode=1, param=0, timing=False):
    """rsgt: [X, Y, Z] receiver SGT stresses (6, knt, npts) or None; ssgt the source SGT.
    mode 0: the reference's FP32 arithmetic; mode 1: FP64 accumulation.  param 0: Vp/Vs
    kernels (SI_ker_sta.F90:1297-1298); param 1: lambda/mu kernels (SI_ker_sta_lamu.F90:
    1299-1300).  Returns
    (6, knt, npts) float64 series (slots X -> 0, 3; Y -> 1, 5; Z -> 2, 4)."""
    s = _f(ssgt)
    _, knt, npts = np.asarray(ssgt).shape
    nt1 = 1 if nt1 is None else int(nt1)
    nt2 = knt if nt2 is None else int(nt2)
    rs = [None if r is None else _f(r) for r in rsgt]
    out = np.zeros(6 * knt * npts, np.float64)
    lam_, mu_ = _f(lam), _f(mu)
    ptrs = [None if r is None else _p(r, C.c_float) for r in rs]
    lib(timing).orc_sgt2scatter3(npts, knt, nt1, nt2, float(dt), _p(lam_, C.c_float), _p(mu_, C.c_float), *ptrs,
                           _p(s, C.c_float), int(mode), int(param), _p(out))
    return out.reshape(6, knt, npts)


def iir(series, b, a, mode):
    """filter (mode 1) / filtfilt (mode 2) of SI_ker_sta along axis 0 of a (nt, ...) array."""
    s = np.asarray(series, np.float64)
    nt = s.shape[0]
    flat = s.reshape(nt, -1)
    out = np.zeros_like(flat)
    b_, a_ = _d(b), _d(a)
    for q in range(flat.shape[1]):
        col = np.ascontiguousarray(flat[:, q])
        o = np.zeros(nt)
        lib().orc_iir(_p(col), nt, int(mode), b_.size, _p(b_), _p(a_), _p(o))
        out[:, q] = o
    return out.reshape(s.shape)


def scatter2kernel(v, u, ka, kb, dt, nt1, nt2, sgt_m0, mode=1):
    """Window kernels (phase_Vp, amplitude_Vp, phase_Vs, amplitude_Vs) of series ka, kb
    ((knt, npts) float64) against V and U over frames nt1..nt2 (1-based)."""
    ka_ = np.ascontiguousarray(ka, np.float64)
    kb_ = np.ascontiguousarray(kb, np.float64)
    knt, npts = ka_.shape
    v_, u_ = _f(v), _f(u)
    outs = [np.zeros(npts, np.float64) for _ in range(4)]
    lib().orc_scatter2kernel(npts, knt, int(nt1), int(nt2), float(dt), _p(v_, C.c_float), _p(u_, C.c_float),
                             _p(ka_), _p(kb_), float(sgt_m0), int(mode), *[_p(o) for o in outs])
    return tuple(outs)


def scatter2kernel_filtered(v, u, ka, kb, dt, nt1, nt2, sgt_m0, b, a, mode):
    """scatter2kernel after filtering (mode 1 filter, mode 2 filtfilt) of the synthetics V,
    U and of the two series ka, kb along time (SI_ker_sta.F90:756-773), FP64 throughout."""
    fv = _d(iir(np.asarray(v, np.float32).astype(np.float64), b, a, mode))
    fu = _d(iir(np.asarray(u, np.float32).astype(np.float64), b, a, mode))
    fa = _d(iir(ka, b, a, mode))
    fb = _d(iir(kb, b, a, mode))
    knt, npts = np.asarray(ka).shape
    outs = [np.zeros(npts, np.float64) for _ in range(4)]
    lib().orc_scatter2kernel_dv(npts, knt, int(nt1), int(nt2), float(dt), _p(fv), _p(fu), _p(fa), _p(fb),
                                float(sgt_m0), *[_p(o) for o in outs])
    return tuple(outs)


def lsqr(row_ptr, col, val, b, ncol, atol=1e-7, btol=1e-7, maxit=30000, timing=False):
    """slsqr + lgtsol of inv.LSQR/mod_LSQR.f90 on a compressed-row matrix (0-based).
    Returns dict(x, serr, sig, itct, flag, anorm, res2, test1, test2, phibar, xnorm); serr
    for all ncol unknowns."""
    rp = np.ascontiguousarray(row_ptr, np.int64)
    ci = np.ascontiguousarray(col, np.int32)
    va = _d(val)
    b_ = _d(b)
    nrow = rp.size - 1
    x = np.zeros(int(ncol))
    sig = np.zeros(int(ncol))
    info = np.zeros(6)
    flag = C.c_int()
    it = lib(timing).orc_lsqr(nrow, int(ncol), rp.ctypes.data_as(C.POINTER(C.c_longlong)), _p(ci, C.c_int), _p(va), _p(b_),
                        float(atol), float(btol), int(maxit), _p(x), _p(sig), _p(info), C.byref(flag))
    serr = np.zeros(int(ncol))
    lib().orc_lgtsol(nrow, int(ncol), float(info[1]), _p(sig), _p(serr))
    return dict(x=x, serr=serr, sig=sig, itct=int(it), flag=flag.value, anorm=info[0], res2=info[1], test1=info[2],
                test2=info[3], phibar=info[4], xnorm=info[5])


def _fo(a):
    """float32 Fortran-order flattening, or NULL for None"""
    if a is None:
        return None
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, order="F"))


class MediaOracle:
    """CPU restatement of seis3d_media's effmedia_eval, media_extend and media_stept_check,
    with the same set-up methods as `fwant_gb300.Media` (arrays in Fortran index order:
    a[i, j, k])."""

    def __init__(self, ni, nj, nk, x, y, z, ztopo, half_sample=(1, 1, 1), timing=False):
        self._L = lib(timing)
        self.shape = (ni + 6, nj + 6, nk + 6)
        self._keep = [_fo(x), _fo(y), _fo(z)]
        hs = np.ascontiguousarray(half_sample, np.int32)
        self._h = self._L.orc_media_create(ni, nj, nk, *[_p(a, C.c_float) for a in self._keep], float(ztopo),
                                           _p(hs, C.c_int))
        self.result = None

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.orc_media_destroy(self._h)
            self._h = None

    def _fp(self, a):
        a = _fo(a)
        if a is None:
            return None
        self._keep.append(a)
        return _p(a, C.c_float)

    def set_cart1d(self, depth, vp, vs, rho):
        self._L.orc_media_set_cart1d(self._h, len(depth), *[self._fp(a) for a in (depth, vp, vs, rho)])

    def set_layers(self, kind, x, y, z, h, vp, vs, rho, vp_exp=None, vs_exp=None, rho_exp=None):
        ni, nj, nk = np.shape(h)
        self._L.orc_media_set_layers(self._h, int(kind), ni, nj, nk,
                                     *[self._fp(a) for a in (x, y, z, h, vp, vs, rho, vp_exp, vs_exp, rho_exp)])

    def set_volume(self, perturbed, x, y, rz, rz0, vp, vs, rho):
        ni, nj, nk = np.shape(vp)
        self._L.orc_media_set_volume(self._h, int(perturbed), ni, nj, nk, self._fp(x), self._fp(y), self._fp(rz),
                                     float(rz0), self._fp(vp), self._fp(vs), self._fp(rho))

    def set_verpoly(self, perturbed, x, y, rz, rz0, vp_c, vs_c, rho_c, vp_exp, vs_exp, rho_exp):
        ni, nj, nk, npoly = np.shape(vp_c)
        self._L.orc_media_set_verpoly(self._h, int(perturbed), ni, nj, nk, npoly, self._fp(x), self._fp(y),
                                      self._fp(rz), float(rz0),
                                      *[self._fp(a) for a in (vp_c, vs_c, rho_c, vp_exp, vs_exp, rho_exp)])

    def eval(self):
        """(lambda, mu, rho), each (ni+6, nj+6, nk+6) float32, ghosts extended."""
        n = int(np.prod(self.shape))
        outs = [np.zeros(n, np.float32) for _ in range(3)]
        if self._L.orc_media_eval(self._h, *[_p(o, C.c_float) for o in outs]) != 0:
            raise RuntimeError(self._L.orc_media_last_error(self._h).decode())
        self.result = outs
        return tuple(o.reshape(self.shape, order="F") for o in outs)

    def stept_check(self):
        """(dtmax, (i, j, k) 1-based local index, Vp, dL) of the last eval."""
        dt, vp, dl = C.c_float(), C.c_float(), C.c_float()
        ijk = np.zeros(3, np.int32)
        self._L.orc_media_stept_check(self._h, *[_p(o, C.c_float) for o in self.result], C.byref(dt),
                                      _p(ijk, C.c_int), C.byref(vp), C.byref(dl))
        return dt.value, tuple(int(v) for v in ijk), vp.value, dl.value


class Oracle:
    """CPU restatement of seis3d_wave; dbl=True gives the FP64 (-DDataTypeDouble) solver."""

    def __init__(self, ni, nj, nk, stept, free_surface=True, src_surface=True, dbl=False, timing=False):
        self._L = lib(timing)
        self._h = self._L.orc_create(int(ni), int(nj), int(nk), float(stept), int(bool(free_surface)), int(bool(dbl)))
        self._L.orc_set_srcsurface(self._h, int(bool(src_surface)))
        self.ni, self.nj, self.nk = int(ni), int(nj), int(nk)
        self.nx, self.ny, self.nz = self.ni + 6, self.nj + 6, self.nk + 6
        self.shape = (self.nx, self.ny, self.nz)
        self.num_pt = 0

    def close(self):
        if getattr(self, "_h", None):
            self._L.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _keep(self, *a):
        self._refs = a

    def set_coord(self, x, y, z):
        a = [_d(x), _d(y), _d(z)]
        self._L.orc_set_coord(self._h, *[_p(v) for v in a])
        self.x, self.y, self.z = [np.asarray(v, np.float32) for v in (x, y, z)]

    def set_metric(self, xsin, xcot, xi_x, eta_y, zeta_z):
        a = [_d(v) for v in (xsin, xcot, xi_x, eta_y, zeta_z)]
        self._L.orc_set_metric(self._h, *[_p(v) for v in a])

    def compute_metric(self):
        m = metric(self.x, self.y, self.z)
        self.set_metric(m["xsin"], m["xcot"], m["xi_x"], m["eta_y"], m["zeta_z"])

    def set_topography(self, h):
        """Gaussian-hill extension: heights h (nx, ny) in m of the terrain-following radius
        r = z(k) + h s(k); after set_coord and the metric."""
        a = _d(np.asarray(h, np.float32).reshape(-1, order="F"))
        self._L.orc_set_topography(self._h, _p(a))

    def topography_array(self, which):
        """0 r, 1 zeta_r, 2 zeta_theta/r, 3 zeta_phi/(r sin theta) as (nx, ny, nz); 4, 5 the
        surface normal's m1, m2 (nx, ny); 6 the 3x3 inverses (nx, ny, 9)."""
        n2 = self.nx * self.ny
        n = n2 * self.nz if which < 4 else (n2 if which < 6 else 9 * n2)
        out = np.zeros(n)
        self._L.orc_topography_array(self._h, int(which), _p(out))
        if which < 4:
            return out.reshape(self.shape, order="F")
        if which < 6:
            return out.reshape(self.nx, self.ny, order="F")
        return out.reshape(9, self.nx, self.ny, order="F").transpose(1, 2, 0)

    def set_media(self, lam, mu, rho):
        a = [_d(np.asarray(v, np.float32).reshape(-1, order="F")) for v in (lam, mu, rho)]
        self._L.orc_set_media(self._h, *[_p(v) for v in a])

    def set_pml(self, number, velocity, bmax, amax):
        n = np.ascontiguousarray(np.asarray(number, np.int32).reshape(6))
        a = [_d(np.asarray(v, np.float32)) for v in (velocity, bmax, amax)]
        rc = self._L.orc_set_pml(self._h, _p(n, C.c_int), *[_p(v) for v in a])
        if rc:
            raise RuntimeError(self._L.orc_last_error(self._h).decode())

    def set_forces(self, indx, shift, start_time, stf_time, stf_freq, fx, fy, fz, stf_id=200):
        indx = np.ascontiguousarray(np.asarray(indx, np.int32).reshape(-1, 3))
        num = indx.shape[0]
        ntwin = np.asarray(stf_time).size
        a = [_d(np.asarray(shift, np.float32).reshape(-1, 3)), _d(np.asarray(start_time, np.float32)),
             _d(np.asarray(stf_time, np.float32)), _d(np.asarray(stf_freq, np.float32))]
        f = [_d(np.asarray(q, np.float32).reshape(num, ntwin)) for q in (fx, fy, fz)]
        self._L.orc_set_forces(self._h, num, ntwin, _p(indx, C.c_int), *[_p(v) for v in a], *[_p(v) for v in f],
                               int(stf_id))

    def set_moments(self, indx, shift, start_time, stf_time, stf_freq, mom, stf_id=200):
        indx = np.ascontiguousarray(np.asarray(indx, np.int32).reshape(-1, 3))
        num = indx.shape[0]
        ntwin = np.asarray(stf_time).size
        a = [_d(np.asarray(shift, np.float32).reshape(-1, 3)), _d(np.asarray(start_time, np.float32)),
             _d(np.asarray(stf_time, np.float32)), _d(np.asarray(stf_freq, np.float32)),
             _d(np.asarray(mom, np.float32).reshape(6, num, ntwin))]
        self._L.orc_set_moments(self._h, num, ntwin, _p(indx, C.c_int), *[_p(v) for v in a], int(stf_id))

    def set_receivers(self, indx, tinv=1):
        indx = np.ascontiguousarray(np.asarray(indx, np.int32).reshape(-1, 3))
        self.num_pt = indx.shape[0]
        self._L.orc_set_receivers(self._h, self.num_pt, _p(indx, C.c_int), int(tinv))
        self._rec = indx

    def run(self, nsteps):
        if self._L.orc_run(self._h, int(nsteps)):
            raise RuntimeError(self._L.orc_last_error(self._h).decode())

    @property
    def ntime(self):
        return self._L.orc_ntime(self._h)

    @property
    def free_surface(self):
        return bool(self._L.orc_freenode(self._h))

    def get_field(self, component):
        c = COMPONENTS.index(component) if isinstance(component, str) else int(component)
        out = np.zeros(self.nx * self.ny * self.nz)
        self._L.orc_get_field(self._h, c, _p(out))
        return out.reshape(self.shape, order="F")

    def set_field(self, component, values):
        c = COMPONENTS.index(component) if isinstance(component, str) else int(component)
        a = _d(np.asarray(values).reshape(-1, order="F"))
        self._L.orc_set_field(self._h, c, _p(a))

    def pml_profile(self, axis):
        n = (self.nx, self.ny, self.nz)[axis]
        A, B, D = np.zeros(n), np.zeros(n), np.zeros(n)
        self._L.orc_get_pml_profile(self._h, axis, _p(A), _p(B), _p(D))
        return A, B, D

    def get_seismo(self, max_samples=None):
        if max_samples is None:
            max_samples = self.ntime + 1
        out = np.zeros(9 * max(max_samples, 1) * max(self.num_pt, 1))
        n = self._L.orc_get_seismo(self._h, _p(out), int(max_samples))
        return out[: 9 * n * self.num_pt].reshape(9, n, self.num_pt)


def metric(x, y, z, dp=False, full=False):
    """seis3d_metric restated in SP (seis3d_metric.F90:83-112); dp=True evaluates the same
    formula in double from the SP coordinates (the FP64 precomputation); full=True also
    keeps the double results (the metric of the FP64 run) instead of rounding to FP32."""
    x, y, z = [np.ascontiguousarray(np.asarray(v, np.float32)) for v in (x, y, z)]
    if full:
        out = [np.zeros(x.size), np.zeros(x.size), np.zeros(x.size), np.zeros(y.size), np.zeros(z.size)]
        lib().orc_metric_dd(x.size, y.size, z.size, _p(x, C.c_float), _p(y, C.c_float), _p(z, C.c_float),
                            *[_p(v) for v in out])
        return dict(zip(("xsin", "xcot", "xi_x", "eta_y", "zeta_z"), out))
    out = [np.zeros(x.size, np.float32), np.zeros(x.size, np.float32), np.zeros(x.size, np.float32),
           np.zeros(y.size, np.float32), np.zeros(z.size, np.float32)]
    fn = lib().orc_metric_dp if dp else lib().orc_metric
    fn(x.size, y.size, z.size, _p(x, C.c_float), _p(y, C.c_float), _p(z, C.c_float),
       *[_p(v, C.c_float) for v in out])
    return dict(zip(("xsin", "xcot", "xi_x", "eta_y", "zeta_z"), out))


def stf(t, t0, f0, stf_id=200, ntime=1, stept=0.01, dbl=False):
    return lib().orc_stf(0, int(stf_id), t, t0, f0, int(ntime), stept, int(dbl))


def svf(t, t0, f0, stf_id=200, ntime=1, stept=0.01, dbl=False):
    return lib().orc_stf(1, int(stf_id), t, t0, f0, int(ntime), stept, int(dbl))


def norm_delt(x0, y0, z0):
    out = np.zeros(343)
    if lib().orc_norm_delt(x0, y0, z0, _p(out)):
        raise RuntimeError("cal_norm_delt is zero")
    return out.reshape(7, 7, 7, order="F")  # [li, lj, lk]


def pml_R(n):
    return lib().orc_pml_R(int(n))


def op(kind, fwd, f, i):
    """kind 0 DRP/opt, 1 2-4, 2 2-2 one-sided operator on a 1-D array at 0-based i."""
    a = _d(f)
    return lib().orc_op(int(kind), int(bool(fwd)), _p(a), int(i))
