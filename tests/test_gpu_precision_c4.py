"""C4 precision study on the GPU against the FP64 reference run.

For each wavefield storage kind (FP32, BF16, FP16 with FP32 arithmetic) both simulations
of the station pair run on the GPU with device SGT recording, the ZZ kernel is
accumulated on the GPU in FP64, and the relative L2 errors of the velocity seismograms
and of the four kernels against the double-precision CPU run are printed and bounded:
FP32 seismograms and kernels within 1e-4 (the solver's FP32 acceptance bound); BF16 and
FP16 seismograms within the bounds their unit roundoff allows over 1000 steps (random-walk
estimate sqrt(4 * 1000) * u / sqrt(3), times three: BF16 0.43, FP16 0.054); FP16 kernels
within 5e-2.  BF16 kernels are only required to be finite: measured errors of 30-350%
(the kernel correlates two recorded wavefields over their full length, so the rounding
noise of 8-bit significands does not average out) make BF16 storage unfit for kernels.
"""
import os

import numpy as np
import pytest

import c4_study as S

pytestmark = pytest.mark.gpu

REF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c4_fp64_reference.npz")
SEIS_TOL = {"fp32": 1e-4, "bf16": 3 * np.sqrt(4 * S.NT) * 2.0 ** -8 / np.sqrt(3),
            "fp16": 3 * np.sqrt(4 * S.NT) * 2.0 ** -11 / np.sqrt(3)}


def _run(m, storage, scales=None, peak_every=0):
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    st = {"fp32": fw.STORAGE_FP32, "bf16": fw.STORAGE_BF16, "fp16": fw.STORAGE_FP16}[storage]
    s = fw.Solver(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface, storage=st)
    if scales:
        s.set_storage_scale(*scales)
    inputs.attach(s, m)
    s.set_sgt_record(S.SUBS, S.SUBC, S.SUBT, S.TINV, S.KNT)
    peak = np.zeros(9, np.float32)
    if peak_every:
        done = 0
        while done < S.NT:
            n = min(peak_every, S.NT - done)
            s.run(n)
            done += n
            peak = np.maximum(peak, s.max_abs())
    else:
        s.run(S.NT)
    s.check()
    return s, peak


def _scales(peak):
    v, t = float(np.max(peak[:3])), float(np.max(peak[3:]))
    return tuple(float(2.0 ** np.floor(np.log2(8192.0 / x))) for x in (v, t))


@pytest.fixture(scope="module")
def reference():
    if not os.path.exists(REF):
        pytest.skip("FP64 reference fixture not generated (tests/golden/make_c4_reference.py)")
    d = np.load(REF)
    assert int(d["nt"]) == S.NT and int(d["tinv"]) == S.TINV
    return d


@pytest.fixture(scope="module")
def fp16_scales(native_lib):
    ma, mb = S.models()
    peaks = [_run(m, "fp32", peak_every=50)[1] for m in (ma, mb)]
    return _scales(np.maximum(*peaks))


@pytest.mark.parametrize("storage", ["fp32", "bf16", "fp16"])
def test_c4_precision(storage, reference, fp16_scales, native_lib):
    import fwant_gb300 as fw
    ma, mb = S.models()
    scales = fp16_scales if storage == "fp16" else None
    sa, _ = _run(ma, storage, scales)
    sb, _ = _run(mb, storage, scales)
    seis_a = sa.get_seismo()[:3]
    seis_b = sb.get_seismo()[:3]
    errs = {"seis_a": S.rel_l2(seis_a, reference["seis_a"]), "seis_b": S.rel_l2(seis_b, reference["seis_b"])}
    lam, mu = S.block_media(ma)
    kdt, nt1, nt2 = S.window(ma.stept)
    k = fw.SgtKernel(S.NPTS, S.KNT, kdt)
    k.set_media(lam, mu)
    k.take_sgt(2, sb)
    k.take_sgt(3, sa)
    k.scatter(4)
    v, u = S.kernel_waveforms(seis_a[2, :, 1], ma.stept)
    ker = k.kernel(3, v, u, nt1, nt2, S.SGT_M0)
    for name, g, r in zip(("phase_Vp", "amplitude_Vp", "phase_Vs", "amplitude_Vs"), ker, reference["kernels"]):
        errs[name] = S.rel_l2(g, r)
    print(f"C4 {storage}: " + ", ".join(f"{a} {b:.2e}" for a, b in errs.items()) + f" (scatter {k.last_scatter_ms():.1f} ms)")
    for key in ("seis_a", "seis_b"):
        assert errs[key] < SEIS_TOL[storage], (storage, key, errs[key])
    ker_tol = {"fp32": 1e-4, "fp16": 5e-2, "bf16": np.inf}[storage]
    for key in ("phase_Vp", "amplitude_Vp", "phase_Vs", "amplitude_Vs"):
        assert np.isfinite(errs[key]) and errs[key] < ker_tol, (storage, key, errs[key])
