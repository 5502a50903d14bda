"""The medium preprocessor on the GPU against the CPU restatement of seis3d_media
(effmedia_eval, media_extend, media_stept_check), through the C ABI, on seeded models of
every background kind with and without each perturbation kind.

Bit-identical where the evaluation uses only IEEE-rounded +, -, *, / and sqrt (cart1d,
interface, layered and volume backgrounds, volume perturbations): the kernel rounds every
operation separately in the reference's order.  Composite and verpoly models raise samples
to powers through powf, which the device computes within 2 ulp of the host's, so they are
compared to 4e-6 relative."""
import numpy as np
import pytest

import media_case as mc

pytestmark = pytest.mark.gpu

KINDS = [mc.CART1D, mc.INTERFACE, mc.LAYERED, mc.COMPOSITE, mc.VOLUME, mc.VERPOLY]


def _pair(ni, nj, nk, half, kind, perturb, seed=0):
    import fwant_gb300 as fw
    from oracle import oracle as orc
    x, y, z, zt = mc.grid(ni, nj, nk, seed=seed)
    calls = mc.case(kind, x, y, z, zt, seed=seed + 1, perturb=perturb)
    g = mc.feed(fw.Media(ni, nj, nk, x, y, z, zt, half), calls)
    o = mc.feed(orc.MediaOracle(ni, nj, nk, x, y, z, zt, half), calls)
    return g, o


def _compare(g, o, exact):
    got, want = g.eval(), o.eval()
    for a, b, name in zip(got, want, ("lambda", "mu", "rho")):
        assert np.all(np.isfinite(a)), name
        if exact:
            np.testing.assert_array_equal(a, b, err_msg=name)
        else:
            np.testing.assert_allclose(a, b, rtol=4e-6, atol=0, err_msg=name)
    dg, do = g.stept_check(), o.stept_check()
    if exact:
        assert dg == do
    else:
        assert dg[0] == pytest.approx(do[0], rel=4e-6)
    return got


@pytest.mark.parametrize("perturb", [None, mc.VOLUME, mc.VERPOLY])
@pytest.mark.parametrize("kind", KINDS)
def test_model_kinds_match_restatement(kind, perturb, oracle_mod, native_lib):
    exact = kind != mc.COMPOSITE and kind != mc.VERPOLY and perturb != mc.VERPOLY
    g, o = _pair(16, 14, 12, (1, 1, 1), kind, perturb)
    _compare(g, o, exact)


@pytest.mark.parametrize("ni,nj,nk,half", [(33, 5, 7, (2, 1, 0)), (9, 11, 6, (0, 0, 0)), (12, 10, 8, (1, 3, 2))])
def test_shapes_and_sampling(ni, nj, nk, half, oracle_mod, native_lib):
    g, o = _pair(ni, nj, nk, half, mc.INTERFACE, mc.VOLUME, seed=3)
    lam, mu, rho = _compare(g, o, True)
    # ghosts hold the nearest interior value
    c = lambda a, n: np.clip(np.arange(n + 6), 3, n + 2)
    np.testing.assert_array_equal(rho, rho[np.ix_(c(0, ni), c(0, nj), c(0, nk))])


def test_config_sized_grid(oracle_mod, native_lib):
    """100 x 100 x 60 (the CPU-runnable solver configuration), layered background with a
    volume perturbation, two samples per axis: every point bit-identical and a repeat call
    identical"""
    g, o = _pair(100, 100, 60, (1, 1, 1), mc.CART1D, mc.VOLUME, seed=5)
    first = _compare(g, o, True)
    again = g.eval()
    for a, b in zip(first, again):
        np.testing.assert_array_equal(a, b)
    assert g.last_eval_ms() > 0


def test_models_replace_earlier_ones(oracle_mod, native_lib):
    """A second background or perturbation replaces the first (its device arrays freed):
    the result equals a handle given only the later models"""
    import fwant_gb300 as fw
    from oracle import oracle as orc
    x, y, z, zt = mc.grid(12, 10, 8, seed=6)
    first = mc.case(mc.LAYERED, x, y, z, zt, seed=7, perturb=mc.VERPOLY)
    second = mc.case(mc.VOLUME, x, y, z, zt, seed=8, perturb=mc.VOLUME)
    g = mc.feed(fw.Media(12, 10, 8, x, y, z, zt), first + second)
    o = mc.feed(orc.MediaOracle(12, 10, 8, x, y, z, zt), second)
    for a, b in zip(g.eval(), o.eval()):
        np.testing.assert_array_equal(a, b)


def test_stept_check_ties_and_screen(oracle_mod, native_lib):
    """A homogeneous medium on a uniform-in-angle grid gives many points the same or nearly
    the same limit: the FP32 screen keeps every candidate and the exact pass returns the
    reference's first minimum in loop order"""
    import fwant_gb300 as fw
    from oracle import oracle as orc
    x, y, z, zt = mc.grid(20, 16, 10, seed=9)
    d = np.array([0.0, 1e6], np.float32)
    calls = [("set_cart1d", (d, np.full(2, 6000.0, np.float32), np.full(2, 3400.0, np.float32),
                             np.full(2, 2700.0, np.float32)))]
    g = mc.feed(fw.Media(20, 16, 10, x, y, z, zt), calls)
    o = mc.feed(orc.MediaOracle(20, 16, 10, x, y, z, zt), calls)
    _compare(g, o, True)


def test_device_handoff_to_solver(oracle_mod, native_lib):
    """The evaluated medium handed to a solver device to device (fwant_media_device_arrays
    + fwant_set_media_device) gives the solver the same medium as the host arrays through
    fwant_set_media: identical fields after 16 steps"""
    import fwant_gb300 as fw
    from fwant_gb300 import inputs

    from helpers import small_model
    m = small_model("buried")
    zt = float(m.z[3 + m.nk - 1])
    M = mc.feed(fw.Media(m.ni, m.nj, m.nk, m.x, m.y, m.z, zt), mc.case(mc.CART1D, m.x, m.y, m.z, zt, seed=2,
                                                                      perturb=mc.VOLUME))
    lam, mu, rho = M.eval()
    a = inputs.attach(fw.Solver(m.ni, m.nj, m.nk, m.stept), m)
    b = inputs.attach(fw.Solver(m.ni, m.nj, m.nk, m.stept), m)
    M.to_solver(a)
    b.set_media(lam, mu, rho)
    for s in (a, b):
        s.run(16)
    for c in range(9):
        np.testing.assert_array_equal(a.get_field(c), b.get_field(c))
    assert np.any(a.get_field("Vz"))


def test_errors(oracle_mod, native_lib):
    import fwant_gb300 as fw
    from oracle import oracle as orc
    x, y, z, zt = mc.grid(8, 8, 10)
    m = fw.Media(8, 8, 10, x, y, z, zt)
    with pytest.raises(fw.FwantError):  # no background yet
        m.eval()
    with pytest.raises(fw.FwantError):  # no evaluated medium
        m.stept_check()
    with pytest.raises(fw.FwantError):  # a volume needs two samples per axis
        m.set_volume(0, x[:1], y, z[:3], zt, *(np.ones((1, len(y), 3), np.float32),) * 3)
    with pytest.raises(fw.FwantError):
        fw.Media(8, 8, 10, x, y, z, zt, half_sample=(1, 17, 1))
    # a layered model thinner than the grid is deep: the reference stops with "please
    # increase the thickness of the lowest layer"; both report it
    calls = mc.case(mc.LAYERED, x, y, z, zt)
    kind, mx, my, _, h, vp, vs, rho = calls[0][1]
    thin = [("set_layers", (kind, mx, my, None, (h * np.float32(0.2)).astype(np.float32), vp, vs, rho))]
    with pytest.raises(fw.FwantError, match="lowest layer"):
        mc.feed(fw.Media(8, 8, 10, x, y, z, zt), thin).eval()
    with pytest.raises(RuntimeError, match="lowest layer"):
        mc.feed(orc.MediaOracle(8, 8, 10, x, y, z, zt), thin).eval()
