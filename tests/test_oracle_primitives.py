"""Known-answer tests of the oracle's primitives against values evaluated by hand from
the reference's formulas (the reference ships no golden vectors)."""
import math

import numpy as np
import pytest

MCA = dict(m1=-0.30874, c0=-0.6326, p1=1.233, p2=-0.3334, p3=0.04168)  # mod_macdrp.h:19


def test_macdrp_forward_backward_on_linear(oracle_mod):
    """F/B operators of mod_macdrp.h:69-103 on f(i) = i: the weights sum to -6e-5 (kept as
    in the reference) and their first moment is 0.99998."""
    f = np.arange(20, dtype=np.float64)
    s = sum(MCA.values())
    m1 = -MCA["m1"] + MCA["p1"] + 2 * MCA["p2"] + 3 * MCA["p3"]
    assert abs(s - (-6e-5)) < 1e-12 and abs(m1 - 0.99998) < 1e-12
    for i in (5, 10, 13):
        assert oracle_mod.op(0, True, f, i) == pytest.approx(s * i + m1, abs=1e-12)
        assert oracle_mod.op(0, False, f, i) == pytest.approx(-s * i + m1, abs=1e-12)


def test_vlow_operators_exact_on_linear(oracle_mod):
    """2-4 and 2-2 MacCormack operators (mod_macdrp.h:230-268) differentiate linears exactly."""
    f = 3.0 + 0.5 * np.arange(12, dtype=np.float64)
    for kind in (1, 2):
        for fwd in (True, False):
            assert oracle_mod.op(kind, fwd, f, 6) == pytest.approx(0.5, abs=1e-12)


def ricker(t, fc, t0):
    if t <= 0:
        return 0.0
    u = 2 * math.pi * fc * (t - t0)
    return (u * u / 4 - 0.5) * math.exp(-u * u / 4) * math.sqrt(math.pi) / 2


def test_ricker_closed_form_and_derivative(oracle_mod):
    """fun_ricker / fun_ricker_deriv (mod_src.F90:509-530): closed form, zero for t <= 0,
    and the SVF is the time derivative of the STF."""
    fc, t0 = 0.2, 7.5
    for t in (0.3, 3.0, 7.5, 9.1, 14.0):
        assert oracle_mod.stf(t, t0, fc, dbl=True) == pytest.approx(ricker(t, fc, t0), rel=1e-12, abs=1e-15)
        h = 1e-5
        num = (ricker(t + h, fc, t0) - ricker(t - h, fc, t0)) / (2 * h)
        assert oracle_mod.svf(t, t0, fc, dbl=True) == pytest.approx(num, rel=1e-6, abs=1e-9)
    assert oracle_mod.stf(-1.0, t0, fc) == 0.0 and oracle_mod.stf(0.0, t0, fc) == 0.0
    assert oracle_mod.stf(t0, t0, fc) == pytest.approx(-0.5 * math.sqrt(math.pi) / 2, rel=1e-6)
    # FP32 evaluation stays within float rounding of the double one
    for t in (2.0, 6.0, 8.0):
        assert oracle_mod.stf(t, t0, fc) == pytest.approx(oracle_mod.stf(t, t0, fc, dbl=True), rel=2e-6, abs=1e-7)


def test_other_stf_ids(oracle_mod):
    """gauss (220), bell (230), bell_int (100), triangle (110 svf), step (240), delta (250)."""
    assert oracle_mod.stf(0.5, 1.0, 0.3, stf_id=220, dbl=True) == pytest.approx(
        math.exp(-(0.5 - 1.0) ** 2 / 0.09) / (math.sqrt(math.pi) * 0.3), rel=1e-12)
    assert oracle_mod.stf(2.5, 0.0, 1.0, stf_id=220, dbl=True) == pytest.approx(
        math.exp(-6.25) / math.sqrt(math.pi), rel=1e-12)   # t0 = 0: no window
    assert oracle_mod.stf(0.25, 0.0, 1.0, stf_id=230, dbl=True) == pytest.approx(1 - math.cos(math.pi / 2), rel=1e-12)
    assert oracle_mod.stf(2.0, 0.0, 1.0, stf_id=100, dbl=True) == 1.0
    assert oracle_mod.svf(0.25, 0.0, 1.0, stf_id=110, dbl=True) == pytest.approx(0.25 / 0.25, rel=1e-12)
    assert oracle_mod.stf(5.0, 0.0, 1.0, stf_id=240) == 1.0
    assert oracle_mod.stf(0.0, 0.0, 1.0, stf_id=250, ntime=0, stept=0.01, dbl=True) == pytest.approx(100.0)
    assert oracle_mod.stf(0.0, 0.0, 1.0, stf_id=250, ntime=3, stept=0.01) == 0.0
    assert math.isnan(oracle_mod.stf(1.0, 0.0, 1.0, stf_id=999))


def test_norm_delt(oracle_mod):
    """cal_norm_delt (mod_src.F90:419-437): unit sum, symmetric and peaked at the node for a
    zero shift; the peak follows the shift."""
    d = oracle_mod.norm_delt(0.0, 0.0, 0.0)
    assert d.sum() == pytest.approx(1.0, abs=1e-6)
    assert np.allclose(d, d[::-1, :, :]) and np.allclose(d, d.transpose(1, 0, 2)) and np.allclose(d, d.transpose(2, 1, 0))
    assert np.unravel_index(np.argmax(d), d.shape) == (3, 3, 3)
    e = oracle_mod.norm_delt(0.4, -0.3, 0.0)
    assert e.sum() == pytest.approx(1.0, abs=1e-6)
    assert e[4, 3, 3] > e[2, 3, 3] and e[3, 2, 3] > e[3, 4, 3]
    g = np.exp(-(np.arange(-3, 4) / 1.5) ** 2)
    ref = np.einsum("i,j,k->ijk", g, g, g)
    assert np.allclose(d, ref / ref.sum(), rtol=2e-6)


def test_pml_reflection_coefficient(oracle_mod):
    """cal_pml_R (mod_abs_npml.F90:9120-9124)."""
    for n in (4, 8, 12, 20):
        assert oracle_mod.pml_R(n) == pytest.approx(10 ** (-(math.log10(n) - 1) / math.log10(2) - 3), rel=1e-6)


def test_pml_profiles(oracle_mod):
    """abs_init profiles (mod_abs_npml.F90:198-284): d = dmax (x/L)^2 stored as d/b,
    a = amax (1 - x/L), b = 1 + (bmax-1)(x/L)^2; zero damping outside the layers."""
    from fwant_gb300 import inputs
    m = inputs.make_model(30, 26, 22, seed=1, npml=6)
    o = oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept)
    o.set_coord(m.x, m.y, m.z)
    o.set_pml(m.pml_number, m.pml_velocity, m.pml_bmax, m.pml_amax)
    A, B, D = o.pml_profile(0)
    ni1, n = 3, 6
    amax, bmax = float(m.pml_amax[0]), float(m.pml_bmax[0])
    L0 = float(m.z[-4]) * (float(m.x[ni1 + n]) - float(m.x[ni1]))
    R = oracle_mod.pml_R(n)
    dmax = -8000.0 / 2 / L0 * math.log(R) * 3
    for i in range(ni1, ni1 + n + 1):
        q = float(m.z[-4]) * (float(m.x[ni1 + n]) - float(m.x[i])) / L0
        b = 1 + (bmax - 1) * q * q
        assert A[i] == pytest.approx(amax * (1 - q), rel=1e-5, abs=1e-6)
        assert B[i] == pytest.approx(b, rel=1e-5)
        assert D[i] == pytest.approx(dmax * q * q / b, rel=1e-4, abs=1e-6)
    mid = (m.ni + 6) // 2
    assert A[mid] == 0 and B[mid] == 1 and D[mid] == 0
    assert not o.free_surface or m.pml_number[5] == 0


def test_metric_uniform_grid(oracle_mod):
    """seis3d_metric on a uniform axis: x_xi = 0.99998 h (the -6e-5 weight sums of the F and B
    operators cancel in the average)."""
    h = 0.25
    x = (1.0 + h * np.arange(20)).astype(np.float32)
    y = x.copy()
    z = (6.0e6 + 1000.0 * np.arange(20)).astype(np.float32)
    for dp in (True, False):
        met = oracle_mod.metric(x, y, z, dp=dp)
        assert met["xi_x"][3:-3] == pytest.approx(1.0 / (0.99998 * h), rel=1e-5)
        assert met["zeta_z"][3:-3] == pytest.approx(1.0 / (0.99998 * 1000.0), rel=2e-3 if not dp else 1e-6)
        assert met["xi_x"][0] == met["xi_x"][3] and met["xi_x"][-1] == met["xi_x"][-4]
        assert met["xsin"] == pytest.approx(np.sin(x.astype(np.float64)), rel=1e-6)
