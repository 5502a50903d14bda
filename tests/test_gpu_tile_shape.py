"""The stage kernel's tall tile (32 x 16 columns, fwant_set_tile_rows(16)) against the oracle
and against the default 32 x 8 tile:

* the reference-order form with the tall tile reproduces the FP32 oracle bit for bit on
  every boundary path (free surface, buried and surface forces, moment tensor, six-face
  PML, fluid layer), one step of each F/B variant at a time, and on ragged grids;
* the fast form with the tall tile agrees with the default tile to FP32 rounding (the two
  instantiations contract multiply-adds independently), batched or alone;
* the setting is refused where the tall tile does not exist (2-byte storage, a terrain-
  following grid, a batch of mixed shapes), and the autotuner records the shape it keeps.
"""
import numpy as np
import pytest

from helpers import feed, interior, rel_l2, small_model

pytestmark = pytest.mark.gpu

KINDS = ["surface", "buried", "nofree", "moment", "water"]


def _solver(m, met, kind, exact, rows):
    import fwant_gb300 as fw
    s = fw.Solver(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface, exact_arith=exact)
    s.tile_rows = rows
    return feed(s, m, met, kind)


@pytest.mark.parametrize("kind", KINDS)
def test_tall_tile_exact_is_the_oracle(kind, oracle_mod, native_lib):
    m = small_model(kind, nj=37)
    met = oracle_mod.metric(m.x, m.y, m.z)
    g = _solver(m, met, kind, True, 16)
    assert g.tile_rows == 16
    o = feed(oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface), m, met, kind)
    for step in range(1, 9):  # every operator variant and RK stage
        g.run(1)
        o.run(1)
        for c in range(9):
            a, b = interior(g.get_field(c)), interior(o.get_field(c)).astype(np.float32)
            assert np.array_equal(a, b), f"{kind} step {step} component {c}: {int(np.sum(a != b))} values differ"
    g.run(24)
    o.run(24)
    assert np.array_equal(g.get_seismo(), o.get_seismo().astype(np.float32))
    g.close()


@pytest.mark.parametrize("shape", [(33, 19, 21), (40, 9, 30), (64, 41, 9)])
def test_tall_tile_ragged_grids(shape, oracle_mod, native_lib):
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    ni, nj, nk = shape
    m = inputs.make_model(ni, nj, nk, seed=5, npml=3, nrecv=3, source="buried", fc=2.0, t0=0.6)
    met = oracle_mod.metric(m.x, m.y, m.z)
    g = fw.Solver(ni, nj, nk, m.stept, exact_arith=True)
    g.tile_rows = 16
    inputs.attach(g, m, metric=met)
    o = inputs.attach(oracle_mod.Oracle(ni, nj, nk, m.stept), m, metric=met)
    g.run(12)
    o.run(12)
    for c in range(9):
        assert np.array_equal(interior(g.get_field(c)), interior(o.get_field(c)).astype(np.float32)), (shape, c)
    g.close()


def test_tall_tile_fast_form_and_batch(oracle_mod, native_lib):
    import fwant_gb300 as fw
    kinds = ("buried", "surface", "moment")
    models = [small_model(k, nj=30, seed=7) for k in kinds]
    mets = [oracle_mod.metric(m.x, m.y, m.z) for m in models]
    ref = [_solver(m, met, k, False, 8) for m, met, k in zip(models, mets, kinds)]
    alone = [_solver(m, met, k, False, 16) for m, met, k in zip(models, mets, kinds)]
    batched = [_solver(m, met, k, False, 16) for m, met, k in zip(models, mets, kinds)]
    for s in ref + alone:
        s.run(40)
    b = fw.Batch(batched)
    b.run(40)
    for r, a, q in zip(ref, alone, batched):
        for c in range(9):
            x = interior(r.get_field(c))
            if np.any(x):
                assert rel_l2(interior(a.get_field(c)), x) < 1e-6
                assert rel_l2(interior(q.get_field(c)), x) < 1e-6
        assert rel_l2(q.get_seismo(), a.get_seismo()) < 1e-6
    for s in ref + alone + batched:
        s.close()


def test_tall_tile_refusals_and_autotune(oracle_mod, native_lib):
    import fwant_gb300 as fw
    m = small_model("buried")
    met = oracle_mod.metric(m.x, m.y, m.z)
    s16 = fw.Solver(m.ni, m.nj, m.nk, m.stept, storage=fw.STORAGE_BF16)
    with pytest.raises(fw.FwantError):
        s16.tile_rows = 16
    with pytest.raises(fw.FwantError):
        s16.tile_rows = 12
    s16.close()
    a = _solver(m, met, "buried", False, 16)
    c = _solver(m, met, "buried", False, 8)
    with pytest.raises(fw.FwantError):
        fw.Batch([a, c])
    with pytest.raises(fw.FwantError):
        a.set_topography(np.zeros((m.ni + 6, m.nj + 6), np.float32))
    planes = c.autotune(2)
    assert c.tile_rows in (8, 16) and planes >= 3
    c.run(8)
    assert np.all(np.isfinite(c.get_field(0)))
    a.close()
    c.close()
