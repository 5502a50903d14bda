"""Host-side input construction mirrors the reference preprocessors."""
import numpy as np
import pytest

from fwant_gb300 import inputs


def test_grid_ghosts_extrapolate_linearly():
    """read_grid_coord (seis3d_grid.F90:137-147): ghosts continue the edge spacing."""
    g = inputs.grid_coords(10, 0.01, 45.0, None, 1.0, degrees=True)
    assert g.dtype == np.float32 and g.size == 16
    d = np.diff(g.astype(np.float64))
    # FP32 colatitudes near 0.79 rad resolve a 1.7e-4 rad spacing only to ~1e-3
    assert np.allclose(d, d[5], rtol=2e-3)
    assert g[3] == pytest.approx(np.deg2rad(45.0), rel=1e-7)


def test_explicit_z_list_and_stretching():
    zl = inputs.stretched_depths_km(40, 0.5, 2.0)
    h = -np.diff(zl[::-1].astype(np.float64))
    assert h[0] == pytest.approx(0.5, rel=1e-4) and h[-1] == pytest.approx(2.0, rel=1e-4)
    assert np.all(np.diff(h) > 0)
    z = inputs.grid_coords(40, None, 0.0, zl, 1000.0, degrees=False)
    assert z[-4] == pytest.approx(6371.0e3, rel=1e-7)
    assert np.all(np.diff(z) > 0)


def test_locate_and_shift():
    """seis3d_source.F90:100-116: nearest node (first minimum) and fractional shift."""
    c = np.array([0.0, 1.0, 2.0, 3.0, 4.0], np.float32)
    assert inputs.locate(c, 2.4) == 3
    assert inputs.source_shift(c, 3, 2.4) == pytest.approx(0.4, rel=1e-6)
    assert inputs.source_shift(c, 3, 1.7) == pytest.approx(-0.3, rel=1e-5)


def test_model_c1_shapes_and_physics():
    m = inputs.make_model(40, 36, 30, seed=2, npml=6)
    assert m.lam.shape == (46, 42, 36)
    vp = np.sqrt((m.lam + 2 * m.mu) / m.rho)
    vs = np.sqrt(m.mu / m.rho)
    assert 5700 < vp.min() and vp.max() < 8100
    assert np.allclose(vp / vs, 1.73, rtol=1e-3)
    assert m.stept == pytest.approx(0.5 * 500.0 / vp.max(), rel=0.02)
    assert list(m.pml_number) == [6, 6, 6, 6, 6, 0]
    assert np.all(m.recv_indx[:, 2] == 30 + 3)
    assert m.force_indx[0, 2] == 33  # surface force on k = nk2 (1-based)
