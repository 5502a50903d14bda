"""The oracle's terrain-following grid (the Gaussian-hill extension; no counterpart in
the reference, whose grid is orthogonal spherical with a flat top): a zero hill agrees
with the flat restatement to rounding, the FP32 and FP64 restatements agree on a 2 km
hill, and the metric arrays have the expected form."""
import numpy as np

from topo_case import LENFD, hill_model, rel


def _run(O, m, h, steps, dbl=False, metric=None):
    from fwant_gb300 import inputs
    o = O.Oracle(m.ni, m.nj, m.nk, m.stept, dbl=dbl)
    inputs.attach(o, m, metric=metric)
    if h is not None:
        o.set_topography(h)
    o.run(steps)
    return o


def test_zero_hill_equals_the_flat_restatement(oracle_mod):
    m, h = hill_model()
    met = oracle_mod.metric(m.x, m.y, m.z, dp=True)
    flat = _run(oracle_mod, m, None, 120, metric=met)
    zero = _run(oracle_mod, m, np.zeros_like(h), 120, metric=met)
    for c in range(9):
        assert rel(zero.get_field(c), flat.get_field(c)) < 3e-6, c
    assert rel(zero.get_seismo(), flat.get_seismo()) < 3e-6


def test_hill_fp32_against_fp64(oracle_mod):
    m, h = hill_model()
    met = oracle_mod.metric(m.x, m.y, m.z, dp=True)
    a = _run(oracle_mod, m, h, 300, metric=met)
    b = _run(oracle_mod, m, h, 300, dbl=True, metric=met)
    for c in range(9):
        f = a.get_field(c)
        assert np.all(np.isfinite(f))
        assert rel(f, b.get_field(c)) < 5e-5, c
    sa, sb = a.get_seismo(), b.get_seismo()
    assert rel(sa[:3], sb[:3]) < 1e-5 and rel(sa[3:], sb[3:]) < 1e-5


def test_terrain_metric(oracle_mod):
    m, h = hill_model()
    met = oracle_mod.metric(m.x, m.y, m.z, dp=True)
    o = oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept)
    from fwant_gb300 import inputs
    inputs.attach(o, m, metric=met)
    o.set_topography(h)
    r, az, bx, by = (o.topography_array(w) for w in range(4))
    k2 = LENFD + m.nk - 1
    # the free surface follows the hill, the bottom ghost plane stays flat
    np.testing.assert_allclose(r[:, :, k2], m.z[k2].astype(np.float64) + h, rtol=0, atol=1.0)
    np.testing.assert_array_equal(r[:, :, 0], np.broadcast_to(m.z[0], r[:, :, 0].shape).astype(np.float32))
    # far from the hill (a few mm of height) the metric is the flat one; zeta_r shrinks
    # under the hill
    assert np.all(az > 0)
    np.testing.assert_allclose(az[0, 0, :], met["zeta_z"].astype(np.float32), rtol=1e-6)
    c = (LENFD + m.ni // 2, LENFD + m.nj // 2)
    assert az[c[0], c[1], k2] < met["zeta_z"][k2]
    # zeta_theta has the sign of -dh/dtheta: positive on the low-theta flank
    assert bx[c[0] - 4, c[1], k2] < 0 < bx[c[0] + 4, c[1], k2]
    m1, m2, minv = o.topography_array(4), o.topography_array(5), o.topography_array(6)
    np.testing.assert_allclose(m1[:, :], bx[:, :, k2] / az[:, :, k2], rtol=1e-6, atol=1e-12)
    assert np.all(np.isfinite(minv))
