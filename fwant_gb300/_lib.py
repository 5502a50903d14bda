"""ctypes binding of the fwant_gb300 C ABI (include/fwant_gb300.h).

`Solver` mirrors the reference solver's set-up sequence (grid -> metric -> media ->
PML -> sources -> receivers -> time loop) with numpy arrays in the reference's
Fortran layouts.  There is no fallback: if the native library is missing or cannot
be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libfwant_gb300.so")

STORAGE_FP32, STORAGE_BF16, STORAGE_FP16, STORAGE_FP64 = 0, 1, 2, 3
STF_RICKER, STF_GAUSS, STF_BELL, STF_STEP, STF_DELTA = 200, 220, 230, 240, 250
SVF_BELL, SVF_TRIANGLE, SVF_GAUSS = 100, 110, 120
COMPONENTS = ("Vx", "Vy", "Vz", "Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz")

STATUS = {
    0: "OK",
    1: "INVALID_ARG",
    2: "OOM",
    3: "CUDA_ERROR",
    4: "NUMERIC_OVERFLOW",
    5: "TIMEOUT",
    6: "STATE",
}

# (name, restype, argtypes); every fwant_* symbol declared in include/fwant_gb300.h
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p
EXPORTS = [
    ("fwant_version", C.c_char_p, []),
    ("fwant_create", C.c_int, [_vp, C.POINTER(_vp)]),
    ("fwant_destroy", None, [_vp]),
    ("fwant_last_error", C.c_char_p, [_vp]),
    ("fwant_set_coord", C.c_int, [_vp, _fp, _fp, _fp]),
    ("fwant_set_metric", C.c_int, [_vp, _fp, _fp, _fp, _fp, _fp]),
    ("fwant_compute_metric", C.c_int, [_vp]),
    ("fwant_set_topography", C.c_int, [_vp, _fp]),
    ("fwant_get_topography_array", C.c_int, [_vp, C.c_int, _fp]),
    ("fwant_get_metric", C.c_int, [_vp, _fp, _fp, _fp, _fp, _fp]),
    ("fwant_metric_arrays", C.c_int, [C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, C.c_int, _fp, _fp, _fp, _fp, _fp]),
    ("fwant_set_media", C.c_int, [_vp, _fp, _fp, _fp]),
    ("fwant_set_pml", C.c_int, [_vp, _ip, _fp, _fp, _fp]),
    ("fwant_set_forces", C.c_int, [_vp, C.c_int, C.c_int, _ip, _fp, _fp, _fp, _fp, _fp, _fp, _fp, C.c_int]),
    ("fwant_set_moments", C.c_int, [_vp, C.c_int, C.c_int, _ip, _fp, _fp, _fp, _fp, _fp, C.c_int]),
    ("fwant_set_receivers", C.c_int, [_vp, C.c_int, _ip, C.c_int]),
    ("fwant_run", C.c_int, [_vp, C.c_int]),
    ("fwant_reference_steps", C.c_int, [C.c_int]),
    ("fwant_source_time_function", C.c_int, [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_float,
                                              _fp]),
    ("fwant_get_ntime", C.c_int, [_vp, _ip]),
    ("fwant_get_seismo", C.c_int, [_vp, _fp, C.c_int, _ip]),
    ("fwant_get_field", C.c_int, [_vp, C.c_int, _fp]),
    ("fwant_set_field", C.c_int, [_vp, C.c_int, _fp]),
    ("fwant_get_snapshot", C.c_int, [_vp, _ip, _ip, _ip, C.c_int, _ip, _fp]),
    ("fwant_get_snapshot_noalloc", C.c_int, [_vp, _ip, _ip, _ip, C.c_int, _ip, _fp]),
    ("fwant_save_checkpoint", C.c_int, [_vp, C.c_char_p]),
    ("fwant_load_checkpoint", C.c_int, [_vp, C.c_char_p]),
    ("fwant_set_sgt_record", C.c_int, [_vp, _ip, _ip, _ip, C.c_int, C.c_int]),
    ("fwant_get_sgt", C.c_int, [_vp, _fp, C.c_int, _ip]),
    ("fwant_sgtker_create", C.c_int, [C.c_longlong, C.c_int, C.c_double, C.c_int, C.POINTER(_vp)]),
    ("fwant_sgtker_destroy", None, [_vp]),
    ("fwant_sgtker_last_error", C.c_char_p, [_vp]),
    ("fwant_sgtker_set_media", C.c_int, [_vp, _fp, _fp]),
    ("fwant_sgtker_set_sgt", C.c_int, [_vp, C.c_int, _fp]),
    ("fwant_sgtker_take_sgt", C.c_int, [_vp, C.c_int, _vp]),
    ("fwant_sgtker_scatter", C.c_int, [_vp, C.c_int, C.c_int, C.c_int]),
    ("fwant_sgtker_set_param", C.c_int, [_vp, C.c_int]),
    ("fwant_sgtker_get_scatter", C.c_int, [_vp, C.c_int, C.POINTER(C.c_double)]),
    ("fwant_sgtker_kernel", C.c_int, [_vp, C.c_int, _fp, _fp, C.c_int, C.c_int, C.c_double,
                                      C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]),
    ("fwant_sgtker_last_scatter_ms", C.c_int, [_vp, C.POINTER(C.c_double)]),
    ("fwant_sgtker_rotate", C.c_int, [_vp, C.POINTER(C.c_double)]),
    ("fwant_sgtker_scatter_pair", C.c_int, [_vp]),
    ("fwant_sgtker_kernel_pair", C.c_int, [_vp, _fp, _fp, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int,
                                           C.POINTER(C.c_double), C.POINTER(C.c_double), _fp, _fp, _fp, _fp]),
    ("fwant_sgtker_convert", C.c_int, [_vp, C.c_int, _fp, _fp, _fp, _fp]),
    ("fwant_sgtker_kernel_filtered", C.c_int, [_vp, C.c_int, _fp, _fp, C.c_int, C.c_int, C.c_double, C.c_int,
                                               C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                               C.POINTER(C.c_double), C.POINTER(C.c_double),
                                               C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("fwant_autotune", C.c_int, [_vp, C.c_int, _ip]),
    ("fwant_batch_autotune", C.c_int, [_vp, C.c_int, _ip]),
    ("fwant_set_planes_per_cta", C.c_int, [_vp, C.c_int]),
    ("fwant_get_planes_per_cta", C.c_int, [_vp, _ip]),
    ("fwant_set_tile_rows", C.c_int, [_vp, C.c_int]),
    ("fwant_get_tile_rows", C.c_int, [_vp, _ip]),
    ("fwant_set_lean_stages", C.c_int, [_vp, C.c_int]),
    ("fwant_check_wait_timeout", C.c_int, [_vp, C.c_int]),
    ("fwant_get_lean_stages", C.c_int, [_vp, _ip]),
    ("fwant_set_rk_scheme", C.c_int, [_vp, C.c_int]),
    ("fwant_get_rk_scheme", C.c_int, [_vp, _ip]),
    ("fwant_batch_create", C.c_int, [C.POINTER(_vp), C.c_int, C.POINTER(_vp)]),
    ("fwant_batch_destroy", None, [_vp]),
    ("fwant_batch_last_error", C.c_char_p, [_vp]),
    ("fwant_batch_set_ctas", C.c_int, [_vp, C.c_int]),
    ("fwant_batch_run", C.c_int, [_vp, C.c_int]),
    ("fwant_batch_last_run_ms", C.c_int, [_vp, C.POINTER(C.c_double)]),
    ("fwant_batch_profile_stages", C.c_int, [_vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("fwant_batch_launches_per_step", C.c_int, [_vp, C.POINTER(C.c_int)]),
    ("fwant_set_storage_scale", C.c_int, [_vp, C.c_float, C.c_float]),
    # surrogate kernels (include/fwant_surrogate.h): device pointers, a stream, cudaError_t
    ("fwant_nn_conv3d_fwd", C.c_int, [_vp, _vp, _vp, _vp] + [C.c_int] * 7 + [_vp]),
    ("fwant_nn_conv3d_bwd", C.c_int, [_vp] * 6 + [C.c_int] * 7 + [_vp]),
    ("fwant_nn_linear_fwd", C.c_int, [_vp] * 4 + [C.c_int] * 3 + [_vp]),
    ("fwant_nn_linear_bwd", C.c_int, [_vp] * 6 + [C.c_int] * 3 + [_vp]),
    ("fwant_nn_lrelu_fwd", C.c_int, [_vp, C.c_longlong, C.c_float, _vp]),
    ("fwant_nn_lrelu_bwd", C.c_int, [_vp, _vp, C.c_longlong, C.c_float, _vp]),
    ("fwant_nn_mse", C.c_int, [_vp] * 5 + [C.c_longlong, _vp]),
    ("fwant_nn_adam", C.c_int, [_vp] * 5 + [C.c_longlong] + [C.c_float] * 5 + [C.c_int, _vp]),
    ("fwant_nn_to_bf16", C.c_int, [_vp, _vp, C.c_longlong, _vp]),
    ("fwant_nn_axpby", C.c_int, [_vp, _vp, C.c_float, _vp, C.c_longlong, _vp]),
    ("fwant_nn_basis_fwd", C.c_int, [_vp, _vp, _vp] + [C.c_int] * 4 + [_vp]),
    ("fwant_nn_basis_bwd", C.c_int, [_vp, _vp, _vp] + [C.c_int] * 4 + [_vp]),
    ("fwant_max_abs", C.c_int, [_vp, _fp]),
    ("fwant_check", C.c_int, [_vp]),
    ("fwant_profile_stages", C.c_int, [_vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("fwant_last_run_ms", C.c_int, [_vp, C.POINTER(C.c_double)]),
    # LSQR inversion solver (include/fwant_lsqr.h)
    ("fwant_lsqr_create", C.c_int, [C.c_longlong, C.c_longlong, C.POINTER(C.c_longlong), C.POINTER(C.c_int),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_void_p)]),
    ("fwant_lsqr_destroy", None, [_vp]),
    ("fwant_lsqr_last_error", C.c_char_p, [_vp]),
    ("fwant_lsqr_solve", C.c_int, [_vp, C.c_double, C.c_double, C.c_longlong, C.POINTER(C.c_longlong)]),
    ("fwant_lsqr_solution", C.c_int, [_vp, C.c_longlong, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("fwant_lsqr_info", C.c_int, [_vp, C.POINTER(C.c_double)]),
    ("fwant_lsqr_multiply", C.c_int, [_vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("fwant_lsqr_last_solve_ms", C.c_int, [_vp, C.POINTER(C.c_double)]),
    # kernel assembly onto inversion blocks (include/fwant_assm.h)
    ("fwant_assm_create", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _fp, C.POINTER(C.c_int),
                                    C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_void_p)]),
    ("fwant_assm_destroy", None, [_vp]),
    ("fwant_assm_last_error", C.c_char_p, [_vp]),
    ("fwant_assm_project", C.c_int, [_vp, C.c_int, C.POINTER(_fp), _fp]),
    ("fwant_assm_project_device", C.c_int, [_vp, C.c_int, C.POINTER(C.c_void_p), _fp]),
    ("fwant_assm_sums", C.c_int, [_vp, _fp]),
    ("fwant_assm_last_ms", C.c_int, [_vp, C.POINTER(C.c_double)]),
    # kernel statistics (include/fwant_kerinfo.h)
    ("fwant_kerinfo_create", C.c_int, [C.c_longlong, _fp, C.c_int, C.POINTER(C.c_void_p)]),
    ("fwant_kerinfo_destroy", None, [_vp]),
    ("fwant_kerinfo_last_error", C.c_char_p, [_vp]),
    ("fwant_kerinfo_add_pick", C.c_int, [_vp, C.POINTER(_fp)]),
    ("fwant_kerinfo_end_event", C.c_int, [_vp, C.c_int, C.c_int]),
    ("fwant_kerinfo_records", C.c_int, [_vp, C.POINTER(C.c_int)]),
    ("fwant_kerinfo_totals", C.c_int, [_vp, _fp, C.POINTER(C.c_int)]),
    ("fwant_kerinfo_record", C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("fwant_kerinfo_last_ms", C.c_int, [_vp, C.POINTER(C.c_double)]),
    # medium preprocessor (include/fwant_media.h)
    ("fwant_media_create", C.c_int, [C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, C.c_float, C.POINTER(C.c_int), C.c_int,
                                     C.POINTER(C.c_void_p)]),
    ("fwant_media_destroy", None, [_vp]),
    ("fwant_media_last_error", C.c_char_p, [_vp]),
    ("fwant_media_set_cart1d", C.c_int, [_vp, C.c_int, _fp, _fp, _fp, _fp]),
    ("fwant_media_set_layers", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int] + [_fp] * 10),
    ("fwant_media_set_volume", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, C.c_float, _fp, _fp,
                                         _fp]),
    ("fwant_media_set_verpoly", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, C.c_float]
     + [_fp] * 6),
    ("fwant_media_eval", C.c_int, [_vp, _fp, _fp, _fp]),
    ("fwant_media_stept_check", C.c_int, [_vp, _fp, C.POINTER(C.c_int), _fp, _fp]),
    ("fwant_media_last_eval_ms", C.c_int, [_vp, C.POINTER(C.c_double)]),
    ("fwant_media_device_arrays", C.c_int, [_vp, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                            C.POINTER(C.c_void_p)]),
    ("fwant_set_media_device", C.c_int, [_vp, _vp, _vp, _vp]),
]


class FwantConfig(C.Structure):
    _fields_ = [
        ("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int),
        ("stept", C.c_double),
        ("free_surface", C.c_int), ("src_surface", C.c_int),
        ("storage", C.c_int), ("device", C.c_int), ("exact_arith", C.c_int),
    ]


class FwantError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_LIB = None


def load_library(path: str | None = None):
    """Load (once) and return the native library; raises if it is absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"native library {p} is missing: build it with `python -m fwant_gb300.build` "
            "(there is no CPU fallback)")
    lib = C.CDLL(p)
    for name, res, args in EXPORTS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def _f32(a, n=None):
    """Flatten in C order (callers shape arrays so that C order is the Fortran layout)."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _fortran3(a, shape):
    a = np.asarray(a, dtype=np.float32)
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return np.ascontiguousarray(a.reshape(-1, order="F"))


def _ptr(a, t=C.c_float):
    return a.ctypes.data_as(C.POINTER(t))


class Solver:
    """One simulation on one GPU (the reference's per-rank solver state)."""

    def __init__(self, ni, nj, nk, stept, free_surface=True, src_surface=True, storage=STORAGE_FP32, device=0,
                 exact_arith=False):
        self._lib = load_library()
        cfg = FwantConfig(int(ni), int(nj), int(nk), float(stept), int(bool(free_surface)),
                          int(bool(src_surface)), int(storage), int(device), int(bool(exact_arith)))
        h = C.c_void_p()
        rc = self._lib.fwant_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise FwantError(rc, "fwant_create failed")
        self._h = h
        self.ni, self.nj, self.nk = int(ni), int(nj), int(nk)
        self.nx, self.ny, self.nz = self.ni + 6, self.nj + 6, self.nk + 6
        self.shape = (self.nx, self.ny, self.nz)
        self.stept = float(stept)
        self.num_pt = 0

    def _chk(self, rc):
        if rc != 0:
            raise FwantError(rc, self._lib.fwant_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fwant_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- inputs -----------------------------------------------------------
    def set_coord(self, x, y, z):
        x, y, z = _f32(x, self.nx), _f32(y, self.ny), _f32(z, self.nz)
        self._chk(self._lib.fwant_set_coord(self._h, _ptr(x), _ptr(y), _ptr(z)))

    def set_metric(self, xsin, xcot, xi_x, eta_y, zeta_z):
        a = [_f32(xsin, self.nx), _f32(xcot, self.nx), _f32(xi_x, self.nx), _f32(eta_y, self.ny),
             _f32(zeta_z, self.nz)]
        self._chk(self._lib.fwant_set_metric(self._h, *[_ptr(v) for v in a]))

    def compute_metric(self):
        self._chk(self._lib.fwant_compute_metric(self._h))

    def get_metric(self):
        out = [np.zeros(self.nx, np.float32), np.zeros(self.nx, np.float32), np.zeros(self.nx, np.float32),
               np.zeros(self.ny, np.float32), np.zeros(self.nz, np.float32)]
        self._chk(self._lib.fwant_get_metric(self._h, *[_ptr(v) for v in out]))
        return dict(zip(("xsin", "xcot", "xi_x", "eta_y", "zeta_z"), out))

    def set_media(self, lam, mu, rho):
        a = [_fortran3(v, self.shape) for v in (lam, mu, rho)]
        self._chk(self._lib.fwant_set_media(self._h, *[_ptr(v) for v in a]))

    def set_pml(self, number, velocity, bmax, amax):
        n = np.ascontiguousarray(np.asarray(number, dtype=np.int32).reshape(6))
        v, b, a = (_f32(q, 6) for q in (velocity, bmax, amax))
        self._chk(self._lib.fwant_set_pml(self._h, _ptr(n, C.c_int), _ptr(v), _ptr(b), _ptr(a)))

    def set_forces(self, indx, shift, start_time, stf_time, stf_freq, fx, fy, fz, stf_id=STF_RICKER):
        indx = np.ascontiguousarray(np.asarray(indx, dtype=np.int32).reshape(-1, 3))
        num = indx.shape[0]
        stf_time = _f32(stf_time)
        ntwin = stf_time.size
        args = [_f32(np.asarray(shift).reshape(-1, 3), 3 * num), _f32(start_time, num), stf_time,
                _f32(stf_freq, ntwin)]
        # Fx etc. are (ntwin, num) column-major: index m + ntwin*n
        f = [_f32(np.asarray(q, dtype=np.float32).reshape(num, ntwin), ntwin * num) for q in (fx, fy, fz)]
        self._chk(self._lib.fwant_set_forces(self._h, num, ntwin, _ptr(indx, C.c_int), *[_ptr(q) for q in args],
                                             *[_ptr(q) for q in f], int(stf_id)))

    def set_moments(self, indx, shift, start_time, stf_time, stf_freq, mom, stf_id=STF_RICKER):
        """mom: array (6, num, ntwin) of Mxx Myy Mzz Mxy Mxz Myz."""
        indx = np.ascontiguousarray(np.asarray(indx, dtype=np.int32).reshape(-1, 3))
        num = indx.shape[0]
        stf_time = _f32(stf_time)
        ntwin = stf_time.size
        mom = _f32(np.asarray(mom, dtype=np.float32).reshape(6, num, ntwin), 6 * num * ntwin)
        args = [_f32(np.asarray(shift).reshape(-1, 3), 3 * num), _f32(start_time, num), stf_time,
                _f32(stf_freq, ntwin), mom]
        self._chk(self._lib.fwant_set_moments(self._h, num, ntwin, _ptr(indx, C.c_int), *[_ptr(q) for q in args],
                                              int(stf_id)))

    def set_receivers(self, indx, tinv=1):
        indx = np.ascontiguousarray(np.asarray(indx, dtype=np.int32).reshape(-1, 3))
        self.num_pt = indx.shape[0]
        self._chk(self._lib.fwant_set_receivers(self._h, self.num_pt, _ptr(indx, C.c_int), int(tinv)))

    # --- time loop and outputs ---------------------------------------------
    def run(self, nsteps):
        self._chk(self._lib.fwant_run(self._h, int(nsteps)))

    @property
    def ntime(self):
        v = C.c_int()
        self._chk(self._lib.fwant_get_ntime(self._h, C.byref(v)))
        return v.value

    def last_run_ms(self):
        v = C.c_double()
        self._chk(self._lib.fwant_last_run_ms(self._h, C.byref(v)))
        return v.value

    def profile_stages(self, nsteps):
        """Advance nsteps with per-launch CUDA events; returns (stage_ms[4], step_end_ms)."""
        st = (C.c_double * 4)()
        other = C.c_double()
        self._chk(self._lib.fwant_profile_stages(self._h, int(nsteps), st, C.byref(other)))
        return [st[i] for i in range(4)], other.value

    def get_seismo(self, max_samples=None):
        """Return array (9, nsamp, num_pt)."""
        if max_samples is None:
            max_samples = self.ntime + 1
        out = np.zeros(9 * max(max_samples, 1) * max(self.num_pt, 1), np.float32)
        ns = C.c_int()
        self._chk(self._lib.fwant_get_seismo(self._h, _ptr(out), int(max_samples), C.byref(ns)))
        n = ns.value
        return out[: 9 * n * self.num_pt].reshape(9, n, self.num_pt)

    def set_topography(self, h):
        """Terrain-following grid: heights h (nx, ny) in m, r = z(k) + h s(k) (after the
        coordinates and the metric)."""
        a = _f32(np.asarray(h, np.float32).reshape(-1, order="F"), self.nx * self.ny)
        self._chk(self._lib.fwant_set_topography(self._h, _ptr(a)))

    def topography_array(self, which):
        """0..3: (nx, ny, nz) r, zeta_r, zeta_theta/r, zeta_phi/(r sin theta); 4, 5: the
        surface normal's m1, m2 (nx, ny); 6: the traction-condition inverses (nx, ny, 9)."""
        n2 = self.nx * self.ny
        if which < 4:
            out = np.zeros(n2 * self.nz, np.float32)
            self._chk(self._lib.fwant_get_topography_array(self._h, int(which), _ptr(out)))
            return out.reshape(self.shape, order="F")
        if which < 6:
            out = np.zeros(n2, np.float32)
            self._chk(self._lib.fwant_get_topography_array(self._h, int(which), _ptr(out)))
            return out.reshape(self.nx, self.ny, order="F")
        outs = []
        for e in range(9):
            o = np.zeros(n2, np.float32)
            self._chk(self._lib.fwant_get_topography_array(self._h, 6 + e, _ptr(o)))
            outs.append(o.reshape(self.nx, self.ny, order="F"))
        return np.stack(outs, axis=-1)

    def get_field(self, component):
        c = COMPONENTS.index(component) if isinstance(component, str) else int(component)
        out = np.zeros(self.nx * self.ny * self.nz, np.float32)
        self._chk(self._lib.fwant_get_field(self._h, c, _ptr(out)))
        return out.reshape(self.shape, order="F")

    def set_field(self, component, values):
        c = COMPONENTS.index(component) if isinstance(component, str) else int(component)
        a = _fortran3(values, self.shape)
        self._chk(self._lib.fwant_set_field(self._h, c, _ptr(a)))

    @staticmethod
    def _snap_args(subs, subc, subt, comps):
        comps = [COMPONENTS.index(c) if isinstance(c, str) else int(c) for c in comps]
        a = [np.ascontiguousarray(np.asarray(v, dtype=np.int32).reshape(3)) for v in (subs, subc, subt)]
        cm = np.ascontiguousarray(np.asarray(comps, dtype=np.int32))
        out = np.zeros(int(np.prod(a[1], dtype=np.int64)) * len(comps), np.float32)
        return a, cm, out

    def get_snapshot(self, subs, subc, subt, comps=("Vx", "Vy", "Vz")):
        """Strided sub-volume (1-based subs with ghosts, counts, strides) of the current
        wavefield; returns array (ncomp, nI, nJ, nK) indexed [c, i, j, k]."""
        (s0, c0, t0), cm, out = self._snap_args(subs, subc, subt, comps)
        self._chk(self._lib.fwant_get_snapshot(self._h, _ptr(s0, C.c_int), _ptr(c0, C.c_int), _ptr(t0, C.c_int),
                                               len(cm), _ptr(cm, C.c_int), _ptr(out)))
        return out.reshape(len(cm), int(c0[2]), int(c0[1]), int(c0[0])).transpose(0, 3, 2, 1)

    def get_snapshot_noalloc(self, subs, subc, subt, comps=("Vx", "Vy", "Vz")):
        """get_snapshot through the entry point that allocates no device memory (staging in
        a fixed 16 MiB device array shared by all calls on the device)."""
        (s0, c0, t0), cm, out = self._snap_args(subs, subc, subt, comps)
        self._chk(self._lib.fwant_get_snapshot_noalloc(self._h, _ptr(s0, C.c_int), _ptr(c0, C.c_int),
                                                       _ptr(t0, C.c_int), len(cm), _ptr(cm, C.c_int), _ptr(out)))
        return out.reshape(len(cm), int(c0[2]), int(c0[1]), int(c0[0])).transpose(0, 3, 2, 1)

    def save_checkpoint(self, path):
        self._chk(self._lib.fwant_save_checkpoint(self._h, os.fsencode(path)))

    def load_checkpoint(self, path):
        self._chk(self._lib.fwant_load_checkpoint(self._h, os.fsencode(path)))

    def set_sgt_record(self, subs, subc, subt, tinv, max_frames):
        """Keep sgt_ snapshot frames (six stresses of a strided sub-volume every tinv steps)
        in device memory; subs 1-based with ghosts as in get_snapshot."""
        a = [np.ascontiguousarray(np.asarray(v, dtype=np.int32).reshape(3)) for v in (subs, subc, subt)]
        self._sgt_cnt = tuple(int(v) for v in a[1])
        self._chk(self._lib.fwant_set_sgt_record(self._h, *[_ptr(v, C.c_int) for v in a], int(tinv),
                                                 int(max_frames)))

    def get_sgt(self, max_frames=None):
        """Recorded frames as (6, nframes, npts) float32 (Txx Tyy Tzz Txy Txz Tyz; points i
        fastest over the sub-volume counts)."""
        npts = int(np.prod(self._sgt_cnt))
        if max_frames is None:
            max_frames = self.ntime
        out = np.zeros(6 * max(int(max_frames), 1) * npts, np.float32)
        nf = C.c_int()
        self._chk(self._lib.fwant_get_sgt(self._h, _ptr(out), int(max_frames), C.byref(nf)))
        n = nf.value
        return out[: 6 * n * npts].reshape(6, n, npts)

    def autotune(self, trial_steps=4):
        """Pick the fastest tile shape and planes-per-CTA (before the first step); returns
        the planes (tile_rows reads the shape)."""
        v = C.c_int()
        self._chk(self._lib.fwant_autotune(self._h, int(trial_steps), C.byref(v)))
        return v.value

    @property
    def planes_per_cta(self):
        v = C.c_int()
        self._chk(self._lib.fwant_get_planes_per_cta(self._h, C.byref(v)))
        return v.value

    @planes_per_cta.setter
    def planes_per_cta(self, planes):
        self._chk(self._lib.fwant_set_planes_per_cta(self._h, int(planes)))

    @property
    def tile_rows(self):
        v = C.c_int()
        self._chk(self._lib.fwant_get_tile_rows(self._h, C.byref(v)))
        return v.value

    @tile_rows.setter
    def tile_rows(self, rows):
        self._chk(self._lib.fwant_set_tile_rows(self._h, int(rows)))

    def check_wait_timeout(self, spins=1000):
        """Run the bounded-wait deadline check; raises FwantError (TIMEOUT) as designed."""
        self._chk(self._lib.fwant_check_wait_timeout(self._h, int(spins)))

    @property
    def lean_stages(self):
        """Bit mask of the RK stages split into interior-only and full launches."""
        v = C.c_int()
        self._chk(self._lib.fwant_get_lean_stages(self._h, C.byref(v)))
        return v.value

    @lean_stages.setter
    def lean_stages(self, mask):
        self._chk(self._lib.fwant_set_lean_stages(self._h, int(mask)))

    @property
    def rk_scheme(self):
        """1: the fast FP32 form runs stages 1-3 without t (t formed at stage 3), 0: t
        carried as the reference does (always 0 where the form does not allow 1)."""
        v = C.c_int()
        self._chk(self._lib.fwant_get_rk_scheme(self._h, C.byref(v)))
        return v.value

    @rk_scheme.setter
    def rk_scheme(self, scheme):
        self._chk(self._lib.fwant_set_rk_scheme(self._h, int(scheme)))

    def set_storage_scale(self, velocity_scale, stress_scale):
        """Power-of-two scales of 2-byte storage (stored value = physical value * scale)."""
        self._chk(self._lib.fwant_set_storage_scale(self._h, float(velocity_scale), float(stress_scale)))

    def max_abs(self):
        """Per-component max |value| (receiver order Vx Vy Vz Txx Tyy Tzz Txy Txz Tyz)."""
        out = np.zeros(9, np.float32)
        self._chk(self._lib.fwant_max_abs(self._h, _ptr(out)))
        return out

    def check(self):
        """macdrp_check: raises FwantError(NUMERIC_OVERFLOW) on NaN/Inf/huge."""
        self._chk(self._lib.fwant_check(self._h))


class Batch:
    """Solvers stepped together: one launch per RK stage for up to 16 members."""

    def __init__(self, solvers):
        self._lib = load_library()
        self.solvers = list(solvers)
        arr = (_vp * len(self.solvers))(*[s._h.value for s in self.solvers])
        h = C.c_void_p()
        rc = self._lib.fwant_batch_create(arr, len(self.solvers), C.byref(h))
        if rc != 0:
            raise FwantError(rc, "fwant_batch_create failed")
        self._h = h

    def _chk(self, rc):
        if rc != 0:
            raise FwantError(rc, self._lib.fwant_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fwant_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_ctas(self, ctas):
        self._chk(self._lib.fwant_batch_set_ctas(self._h, int(ctas)))

    def autotune(self, trial_steps=4):
        """Tune every member and the CTA schedule (before the first step); returns ctas."""
        v = C.c_int()
        self._chk(self._lib.fwant_batch_autotune(self._h, int(trial_steps), C.byref(v)))
        return v.value

    def run(self, nsteps):
        self._chk(self._lib.fwant_batch_run(self._h, int(nsteps)))

    def last_run_ms(self):
        ms = C.c_double()
        self._chk(self._lib.fwant_batch_last_run_ms(self._h, C.byref(ms)))
        return ms.value

    def profile_stages(self, nsteps):
        """(average ms of each of the four stage launches, ms of the step-end kernels)."""
        st = (C.c_double * 4)()
        other = C.c_double()
        self._chk(self._lib.fwant_batch_profile_stages(self._h, int(nsteps), st, C.byref(other)))
        return list(st), other.value

    def launches_per_step(self):
        """Kernels one step launches (counted by the last step enqueued)."""
        v = C.c_int()
        self._chk(self._lib.fwant_batch_launches_per_step(self._h, C.byref(v)))
        return v.value


class SgtKernel:
    """Sensitivity-kernel accumulation of one block of npts kernel points
    (SI_ker_sta.F90: stress2strain, sgt2scatter3, scatter2kernel) on the GPU, FP64 sums.
    which: 0/1/2 = receiver station X/Y/Z force SGT, 3 = source station SGT."""

    def __init__(self, npts, knt, kdt, device=0):
        self._lib = load_library()
        h = C.c_void_p()
        rc = self._lib.fwant_sgtker_create(int(npts), int(knt), float(kdt), int(device), C.byref(h))
        if rc != 0:
            raise FwantError(rc, "fwant_sgtker_create failed")
        self._h = h
        self.npts, self.knt, self.kdt = int(npts), int(knt), float(kdt)

    def _chk(self, rc):
        if rc != 0:
            raise FwantError(rc, self._lib.fwant_sgtker_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fwant_sgtker_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_media(self, lam, mu):
        a, b = _f32(lam, self.npts), _f32(mu, self.npts)
        self._chk(self._lib.fwant_sgtker_set_media(self._h, _ptr(a), _ptr(b)))

    def set_sgt(self, which, stress):
        a = _f32(stress, 6 * self.knt * self.npts)
        self._chk(self._lib.fwant_sgtker_set_sgt(self._h, int(which), _ptr(a)))

    def take_sgt(self, which, solver):
        self._chk(self._lib.fwant_sgtker_take_sgt(self._h, int(which), solver._h))

    def set_param(self, param):
        """0: Vp/Vs kernels (SI_ker_sta); 1: lambda/mu kernels (SI_ker_sta_lamu)."""
        self._chk(self._lib.fwant_sgtker_set_param(self._h, int(param)))

    def scatter(self, flags, nt1=1, nt2=None):
        nt2 = self.knt if nt2 is None else int(nt2)
        self._chk(self._lib.fwant_sgtker_scatter(self._h, int(flags), int(nt1), nt2))

    def get_scatter(self, slot):
        out = np.zeros(self.knt * self.npts, np.float64)
        self._chk(self._lib.fwant_sgtker_get_scatter(self._h, int(slot), _ptr(out, C.c_double)))
        return out.reshape(self.knt, self.npts)

    def kernel(self, ncmp, v, u, nt1, nt2, sgt_m0, filt=None):
        """(phase_Vp, amplitude_Vp, phase_Vs, amplitude_Vs) as float64 arrays of npts.
        filt: None or (mode, b, a) with mode 1 (one pass) or 2 (forward-backward)."""
        v_, u_ = _f32(v, self.knt), _f32(u, self.knt)
        outs = [np.zeros(self.npts, np.float64) for _ in range(4)]
        if filt is None:
            self._chk(self._lib.fwant_sgtker_kernel(self._h, int(ncmp), _ptr(v_), _ptr(u_), int(nt1), int(nt2),
                                                    float(sgt_m0), *[_ptr(o, C.c_double) for o in outs]))
        else:
            mode, b, a = filt
            b_ = np.ascontiguousarray(b, np.float64)
            a_ = np.ascontiguousarray(a, np.float64)
            self._chk(self._lib.fwant_sgtker_kernel_filtered(
                self._h, int(ncmp), _ptr(v_), _ptr(u_), int(nt1), int(nt2), float(sgt_m0), int(mode), int(b_.size),
                _ptr(b_, C.c_double), _ptr(a_, C.c_double), *[_ptr(o, C.c_double) for o in outs]))
        return tuple(outs)

    def rotate(self, rot):
        """Rotate the three force components' series by the 3x3 matrix rot (rot[d, c])."""
        r = np.ascontiguousarray(np.asarray(rot, np.float64).reshape(3, 3).T.reshape(-1))  # column-major
        self._chk(self._lib.fwant_sgtker_rotate(self._h, _ptr(r, C.c_double)))

    def convert(self, mode, kap, kaq, kbp, kbq):
        """Kernel parameter conversion (mode 1 lamu2kamu, 2 lamu2vpvs, 3 vpvs2kamu) of four
        [npts] kernels with the media of set_media; returns the converted four (float32)."""
        arrs = [np.array(np.asarray(x, np.float32).reshape(-1), np.float32) for x in (kap, kaq, kbp, kbq)]
        self._chk(self._lib.fwant_sgtker_convert(self._h, int(mode), *[_ptr(a) for a in arrs]))
        return tuple(arrs)

    def scatter_pair(self):
        """SI_ker_pair's single-precision scatter of the receiver SGT (slot 0) against the
        source SGT (slot 3) over all frames."""
        self._chk(self._lib.fwant_sgtker_scatter_pair(self._h))

    def kernel_pair(self, v, u, nt1, nt2, sgt_m0, mode=0, b=None, a=None):
        """SI_ker_pair's window kernel (FP32): filter mode 0 none, 1 one pass, 2
        forward-backward; returns (Kap, Kaq, Kbp, Kbq) float32 [npts]."""
        vv, uu = _f32(v, self.knt), _f32(u, self.knt)
        nod1 = 0
        bp = ap = None
        if mode:
            bb = np.ascontiguousarray(np.asarray(b, np.float64).reshape(-1))
            aa = np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1))
            nod1 = bb.size
            bp, ap = _ptr(bb, C.c_double), _ptr(aa, C.c_double)
        outs = [np.zeros(self.npts, np.float32) for _ in range(4)]
        self._chk(self._lib.fwant_sgtker_kernel_pair(self._h, _ptr(vv), _ptr(uu), int(nt1), int(nt2),
                                                     float(sgt_m0), int(mode), int(nod1), bp, ap,
                                                     *[_ptr(o) for o in outs]))
        return tuple(outs)

    def last_scatter_ms(self):
        ms = C.c_double()
        self._chk(self._lib.fwant_sgtker_last_scatter_ms(self._h, C.byref(ms)))
        return ms.value


class Lsqr:
    """LSQR on the GPU (inv.LSQR/mod_LSQR.f90: slsqr, lgtsol) for a compressed-row matrix
    (row_ptr, col 0-based, val) and right-hand side b."""

    def __init__(self, row_ptr, col, val, b, ncol, device=0):
        self._lib = load_library()
        rp = np.ascontiguousarray(row_ptr, np.int64)
        ci = np.ascontiguousarray(col, np.int32)
        va = np.ascontiguousarray(val, np.float64)
        bb = np.ascontiguousarray(b, np.float64)
        self.nrow, self.ncol = rp.size - 1, int(ncol)
        if bb.size != self.nrow or ci.size != va.size or ci.size != int(rp[-1]):
            raise ValueError("inconsistent compressed-row arrays")
        h = C.c_void_p()
        rc = self._lib.fwant_lsqr_create(self.nrow, self.ncol, rp.ctypes.data_as(C.POINTER(C.c_longlong)),
                                         _ptr(ci, C.c_int), _ptr(va, C.c_double), _ptr(bb, C.c_double), int(device),
                                         C.byref(h))
        if rc != 0:
            raise FwantError(rc, "fwant_lsqr_create failed")
        self._h = h

    def _chk(self, rc):
        if rc != 0:
            raise FwantError(rc, self._lib.fwant_lsqr_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fwant_lsqr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, atol=1e-7, btol=1e-7, maxit=30000):
        """Iterations run (the reference's defaults)."""
        it = C.c_longlong()
        self._chk(self._lib.fwant_lsqr_solve(self._h, float(atol), float(btol), int(maxit), C.byref(it)))
        return it.value

    def solution(self, nvar=None):
        """(x, standard errors) of the first nvar unknowns (all by default)."""
        n = self.ncol if nvar is None else int(nvar)
        x, e = np.zeros(n), np.zeros(n)
        self._chk(self._lib.fwant_lsqr_solution(self._h, n, _ptr(x, C.c_double), _ptr(e, C.c_double)))
        return x, e

    def info(self):
        v = np.zeros(6)
        self._chk(self._lib.fwant_lsqr_info(self._h, _ptr(v, C.c_double)))
        return dict(zip(("anorm", "res2", "test1", "test2", "phibar", "xnorm"), v))

    def multiply(self, x):
        xx = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.nrow)
        self._chk(self._lib.fwant_lsqr_multiply(self._h, _ptr(xx, C.c_double), _ptr(y, C.c_double)))
        return y

    def last_solve_ms(self):
        ms = C.c_double()
        self._chk(self._lib.fwant_lsqr_last_solve_ms(self._h, C.byref(ms)))
        return ms.value


def _fo(a):
    if a is None:
        return None
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, order="F"))


class Media:
    """The medium preprocessor on the GPU (seis3d_media: effmedia_eval, media_extend,
    media_stept_check).  Grid x[ni+6], y[nj+6], z[nk+6] (radians, metres) with ghosts;
    model arrays in Fortran index order (a[i, j, k], first index fastest)."""

    INTERFACE, LAYERED, COMPOSITE = 2, 3, 4

    def __init__(self, ni, nj, nk, x, y, z, ztopo, half_sample=(1, 1, 1), device=0):
        self._lib = load_library()
        self.shape = (ni + 6, nj + 6, nk + 6)
        self._keep = []
        hs = np.ascontiguousarray(half_sample, np.int32)
        h = C.c_void_p()
        g = [_fo(x), _fo(y), _fo(z)]
        rc = self._lib.fwant_media_create(int(ni), int(nj), int(nk), *[_ptr(a) for a in g], float(ztopo),
                                          _ptr(hs, C.c_int), int(device), C.byref(h))
        if rc != 0:
            raise FwantError(rc, "fwant_media_create failed")
        self._h = h

    def _chk(self, rc):
        if rc != 0:
            raise FwantError(rc, self._lib.fwant_media_last_error(self._h).decode())

    def _fp(self, a):
        a = _fo(a)
        if a is None:
            return None
        self._keep.append(a)
        return _ptr(a)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fwant_media_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_cart1d(self, depth, vp, vs, rho):
        self._chk(self._lib.fwant_media_set_cart1d(self._h, len(depth), *[self._fp(a) for a in (depth, vp, vs, rho)]))

    def set_layers(self, kind, x, y, z, h, vp, vs, rho, vp_exp=None, vs_exp=None, rho_exp=None):
        ni, nj, nk = np.shape(h)
        self._chk(self._lib.fwant_media_set_layers(
            self._h, int(kind), ni, nj, nk, *[self._fp(a) for a in (x, y, z, h, vp, vs, rho, vp_exp, vs_exp, rho_exp)]))

    def set_volume(self, perturbed, x, y, rz, rz0, vp, vs, rho):
        ni, nj, nk = np.shape(vp)
        self._chk(self._lib.fwant_media_set_volume(self._h, int(perturbed), ni, nj, nk, self._fp(x), self._fp(y),
                                                   self._fp(rz), float(rz0), self._fp(vp), self._fp(vs),
                                                   self._fp(rho)))

    def set_verpoly(self, perturbed, x, y, rz, rz0, vp_c, vs_c, rho_c, vp_exp, vs_exp, rho_exp):
        ni, nj, nk, npoly = np.shape(vp_c)
        self._chk(self._lib.fwant_media_set_verpoly(
            self._h, int(perturbed), ni, nj, nk, npoly, self._fp(x), self._fp(y), self._fp(rz), float(rz0),
            *[self._fp(a) for a in (vp_c, vs_c, rho_c, vp_exp, vs_exp, rho_exp)]))

    def eval(self, copy=True):
        """(lambda, mu, rho), each (ni+6, nj+6, nk+6) float32 with ghosts extended; with
        copy=False the medium stays on the device (for stept_check) and None is returned."""
        if not copy:
            self._chk(self._lib.fwant_media_eval(self._h, None, None, None))
            return None
        n = int(np.prod(self.shape))
        outs = [np.zeros(n, np.float32) for _ in range(3)]
        self._chk(self._lib.fwant_media_eval(self._h, *[_ptr(o) for o in outs]))
        return tuple(o.reshape(self.shape, order="F") for o in outs)

    def stept_check(self):
        """(dtmax, (i, j, k) 1-based local index, Vp, dL) of the last eval."""
        dt, vp, dl = C.c_float(), C.c_float(), C.c_float()
        ijk = np.zeros(3, np.int32)
        self._chk(self._lib.fwant_media_stept_check(self._h, C.byref(dt), _ptr(ijk, C.c_int), C.byref(vp),
                                                    C.byref(dl)))
        return dt.value, tuple(int(v) for v in ijk), vp.value, dl.value

    def last_eval_ms(self):
        ms = C.c_double()
        self._chk(self._lib.fwant_media_last_eval_ms(self._h, C.byref(ms)))
        return ms.value

    def to_solver(self, solver):
        """Hand the last evaluated medium to a solver on the same GPU, device to device
        (fwant_media_device_arrays + fwant_set_media_device)."""
        p = [C.c_void_p() for _ in range(3)]
        self._chk(self._lib.fwant_media_device_arrays(self._h, *[C.byref(q) for q in p]))
        solver._chk(self._lib.fwant_set_media_device(solver._h, *p))


def metric(x, y, z, device: int = 0) -> dict:
    """The metric of a grid without a solver (fwant_metric_arrays: seis3d_metric in FP64
    on the device, rounded to FP32): x, y, z with their ghosts in, the arrays of
    metric_mpi*.nc out."""
    x, y, z = (np.ascontiguousarray(np.asarray(a, np.float32)) for a in (x, y, z))
    out = [np.zeros(x.size, np.float32), np.zeros(x.size, np.float32), np.zeros(x.size, np.float32),
           np.zeros(y.size, np.float32), np.zeros(z.size, np.float32)]
    code = load_library().fwant_metric_arrays(x.size - 6, y.size - 6, z.size - 6, _ptr(x), _ptr(y), _ptr(z),
                                              int(device), *[_ptr(v) for v in out])
    if code != 0:
        raise FwantError(code, "fwant_metric_arrays failed")
    return dict(zip(("xsin", "xcot", "xi_x", "eta_y", "zeta_z"), out))


class Assm:
    """Kernel assembly onto inversion blocks on the GPU (SI_ker2assm's projection): the
    block file's volume (max_pix, num_blk), num_of_pix (num_blk) and indx_of_pix
    (3, max_pix, num_blk) in Fortran index order over a kernel volume of shape (ki, kj, kk)."""

    def __init__(self, shape, volume, num_of_pix, indx_of_pix, device=0):
        self._lib = load_library()
        ki, kj, kk = (int(v) for v in shape)
        self.shape = (ki, kj, kk)
        vol = np.asarray(volume, np.float32)
        max_pix, num_blk = vol.shape
        self.num_blk = num_blk
        v = _fo(vol)
        npx = np.ascontiguousarray(np.asarray(num_of_pix, np.int32).reshape(num_blk))
        px = np.ascontiguousarray(np.asarray(indx_of_pix, np.int32).reshape(3, max_pix, num_blk).reshape(-1, order="F"))
        h = C.c_void_p()
        rc = self._lib.fwant_assm_create(ki, kj, kk, num_blk, max_pix, _ptr(v), _ptr(npx, C.c_int), _ptr(px, C.c_int),
                                         int(device), C.byref(h))
        if rc != 0:
            msg = self._lib.fwant_assm_last_error(h).decode() if h.value else "fwant_assm_create failed"
            if h.value:
                self._lib.fwant_assm_destroy(h)
            raise FwantError(rc, msg)
        self._h = h

    def _chk(self, rc):
        if rc != 0:
            raise FwantError(rc, self._lib.fwant_assm_last_error(self._h).decode())

    def project(self, kernels):
        """kernels: 1-4 arrays of shape (ki, kj, kk); returns B (nq, num_blk)."""
        ks = [_fortran3(k, self.shape) for k in kernels]
        arr = (_fp * len(ks))(*[_ptr(k) for k in ks])
        out = np.zeros((len(ks), self.num_blk), np.float32)
        self._chk(self._lib.fwant_assm_project(self._h, len(ks), arr, _ptr(out)))
        return out

    def project_device(self, pointers):
        """Device addresses of 1-4 kernel volumes (Fortran order) on the handle's GPU."""
        arr = (C.c_void_p * len(pointers))(*[int(p) for p in pointers])
        out = np.zeros((len(pointers), self.num_blk), np.float32)
        self._chk(self._lib.fwant_assm_project_device(self._h, len(pointers), arr, _ptr(out)))
        return out

    def sums(self):
        out = np.zeros((4, self.num_blk), np.float32)
        self._chk(self._lib.fwant_assm_sums(self._h, _ptr(out)))
        return out

    def last_ms(self):
        ms = C.c_double()
        self._chk(self._lib.fwant_assm_last_ms(self._h, C.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fwant_assm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class KerInfo:
    """Kernel statistics on the GPU (SI_ker2info's per-point sums, counts and records) over
    volumes of npts points; thresholds kap0 kaq0 kbp0 kbq0."""

    def __init__(self, npts, thresholds, device=0):
        self._lib = load_library()
        self.npts = int(npts)
        th = np.ascontiguousarray(np.asarray(thresholds, np.float32).reshape(4))
        h = C.c_void_p()
        rc = self._lib.fwant_kerinfo_create(self.npts, _ptr(th), int(device), C.byref(h))
        if rc != 0:
            msg = self._lib.fwant_kerinfo_last_error(h).decode() if h.value else "fwant_kerinfo_create failed"
            if h.value:
                self._lib.fwant_kerinfo_destroy(h)
            raise FwantError(rc, msg)
        self._h = h

    def _chk(self, rc):
        if rc != 0:
            raise FwantError(rc, self._lib.fwant_kerinfo_last_error(self._h).decode())

    def add_pick(self, kernels):
        """The four volumes of one pick (any shape of npts points, in point order)."""
        ks = [np.ascontiguousarray(np.asarray(k, np.float32).reshape(self.npts)) for k in kernels]
        arr = (_fp * 4)(*[_ptr(k) for k in ks])
        self._chk(self._lib.fwant_kerinfo_add_pick(self._h, arr))

    def end_event(self, station_tag, event_tag):
        self._chk(self._lib.fwant_kerinfo_end_event(self._h, int(station_tag), int(event_tag)))

    def records(self):
        n = C.c_int()
        self._chk(self._lib.fwant_kerinfo_records(self._h, C.byref(n)))
        return n.value

    def totals(self):
        """(S, N): (4, npts) float32 and int32."""
        S = np.zeros((4, self.npts), np.float32)
        N = np.zeros((4, self.npts), np.int32)
        self._chk(self._lib.fwant_kerinfo_totals(self._h, _ptr(S), _ptr(N, C.c_int)))
        return S, N

    def record(self, r):
        """(M, station tags, event tags) of record r, each (4, npts) int32."""
        out = [np.zeros((4, self.npts), np.int32) for _ in range(3)]
        self._chk(self._lib.fwant_kerinfo_record(self._h, int(r), *[_ptr(o, C.c_int) for o in out]))
        return tuple(out)

    def last_ms(self):
        ms = C.c_double()
        self._chk(self._lib.fwant_kerinfo_last_ms(self._h, C.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fwant_kerinfo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def source_time_function(which: int, stf_id: int, t: float, t0: float, f0: float, ntime: int = 1,
                         stept: float = 0.01) -> float:
    """src_stf (which = 0) or src_svf (which = 1) as the solver tabulates it (host code,
    FP32); raises FwantError for an id the function does not define."""
    out = C.c_float()
    rc = load_library().fwant_source_time_function(int(which), int(stf_id), float(t), float(t0), float(f0),
                                                     int(ntime), float(stept), C.byref(out))
    if rc != 0:
        raise FwantError(rc, f"source time function {stf_id} is not defined for which={which}")
    return float(out.value)


def reference_steps(nt: int) -> int:
    """Steps the reference executes for a configured nt (whole 8-step blocks)."""
    return int(load_library().fwant_reference_steps(int(nt)))
