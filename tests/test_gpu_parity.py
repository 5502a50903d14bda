"""Parity of the CUDA solver with the oracle on seeded small models.

Both sides get identical inputs (coordinates, metric, media, sources), so every field
is compared.  Two arithmetic forms of the same kernel are checked:

* exact_arith=True keeps the reference's FP32 operand order with IEEE division and no
  FMA; it must agree with the oracle to within 1e-6 relative L2 per field (in practice
  it is bit-identical);
* the default fast form (FMA, precomputed reciprocals) must agree within 1e-5 relative
  L2 after 75 steps (the drop-in's tolerance for full runs: 1e-4 on seismograms).
"""
import numpy as np
import pytest

from helpers import feed, interior, rel_l2, small_model

pytestmark = pytest.mark.gpu

KINDS = ["surface", "buried", "nofree", "moment", "water"]


def _pair(kind, oracle_mod, exact):
    import fwant_gb300 as fw
    m = small_model(kind)
    met = oracle_mod.metric(m.x, m.y, m.z)
    g = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface, exact_arith=exact), m, met, kind)
    o = feed(oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface), m, met, kind)
    return m, g, o


@pytest.mark.parametrize("kind", KINDS)
def test_exact_each_step_of_one_cycle(kind, oracle_mod, native_lib):
    """All eight F/B variants and all four RK stages, one step at a time."""
    m, g, o = _pair(kind, oracle_mod, True)
    worst = 0.0
    nonzero = 0
    for step in range(1, 9):
        g.run(1)
        o.run(1)
        for c in range(9):
            a = interior(g.get_field(c))
            b = interior(o.get_field(c))
            if not np.any(b):
                assert not np.any(a), f"{kind} step {step} comp {c}: expected zeros"
                continue
            nonzero += 1
            e = rel_l2(a, b)
            worst = max(worst, e)
            assert e < 1e-6, f"{kind}: step {step} component {c} rel L2 {e:.3e}"
    assert nonzero > 0
    print(f"{kind}: worst rel L2 over 8 steps = {worst:.3e}")


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
@pytest.mark.parametrize("kind", KINDS)
def test_long_run_fields_and_seismograms(kind, exact, oracle_mod, native_lib):
    m, g, o = _pair(kind, oracle_mod, exact)
    # 75 steps: whole 8-step blocks through the CUDA graph plus an eager remainder
    g.run(40)
    g.run(35)
    o.run(75)
    assert g.ntime == o.ntime == 75
    tol = 1e-6 if exact else 1e-5
    for c in range(9):
        a, b = interior(g.get_field(c)), interior(o.get_field(c))
        if np.any(b):
            assert rel_l2(a, b) < tol, f"{kind} component {c}: {rel_l2(a, b):.3e}"
    sg, so = g.get_seismo(), o.get_seismo()
    assert sg.shape == so.shape == (9, 75, m.recv_indx.shape[0])
    for c in range(9):
        if np.any(so[c]):
            assert rel_l2(sg[c], so[c]) < tol, f"{kind} seismogram component {c}: {rel_l2(sg[c], so[c]):.3e}"


def test_exact_is_bitwise(oracle_mod, native_lib):
    """The reference-order form reproduces the FP32 CPU restatement bit for bit."""
    m, g, o = _pair("buried", oracle_mod, True)
    g.run(16)
    o.run(16)
    for c in range(9):
        a, b = g.get_field(c), o.get_field(c).astype(np.float32)
        assert np.array_equal(interior(a), interior(b)), f"component {c}"
    assert np.array_equal(g.get_seismo(), o.get_seismo().astype(np.float32))


def test_run_in_pieces_equals_one_run(oracle_mod, native_lib):
    import fwant_gb300 as fw
    m = small_model("buried")
    met = oracle_mod.metric(m.x, m.y, m.z)
    a = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept), m, met, "buried")
    b = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept), m, met, "buried")
    a.run(27)
    for n in (3, 8, 5, 11):
        b.run(n)
    for c in range(9):
        assert np.array_equal(a.get_field(c), b.get_field(c))
    assert np.array_equal(a.get_seismo(), b.get_seismo())


@pytest.mark.parametrize("shape", [(33, 19, 21), (40, 9, 30), (64, 24, 9)])
def test_ragged_tiles(shape, oracle_mod, native_lib):
    """Grid sizes that are not multiples of the 32 x 8 tile or of the k chunk."""
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    ni, nj, nk = shape
    m = inputs.make_model(ni, nj, nk, seed=5, npml=3, nrecv=3, source="buried", fc=2.0, t0=0.6)
    met = oracle_mod.metric(m.x, m.y, m.z)
    g = inputs.attach(fw.Solver(ni, nj, nk, m.stept, exact_arith=True), m, metric=met)
    o = inputs.attach(oracle_mod.Oracle(ni, nj, nk, m.stept), m, metric=met)
    g.run(12)
    o.run(12)
    for c in range(9):
        b = interior(o.get_field(c))
        if np.any(b):
            assert rel_l2(interior(g.get_field(c)), b) < 1e-6, (shape, c)


def test_fp64_metric(oracle_mod, native_lib):
    """fwant_compute_metric (FP64 on the device) against the same formula evaluated in
    double on the host (1 ulp of FP32 allowed for summation order), and against
    seis3d_metric's SP arithmetic, whose cancellation error on FP32 colatitudes near
    0.87 rad with 1.6e-4 rad spacing reaches ~1e-3 relative."""
    import fwant_gb300 as fw
    m = small_model("surface")
    s = fw.Solver(m.ni, m.nj, m.nk, m.stept)
    s.set_coord(m.x, m.y, m.z)
    s.compute_metric()
    got = s.get_metric()
    ref = oracle_mod.metric(m.x, m.y, m.z, dp=True)
    for k in ref:
        np.testing.assert_allclose(got[k], ref[k], rtol=2.5e-7, err_msg=k)
    sp = oracle_mod.metric(m.x, m.y, m.z)
    for k in sp:
        np.testing.assert_allclose(got[k], sp[k], rtol=2e-3, err_msg=k)


def test_overflow_check_reports_nan(native_lib):
    """macdrp_check: a NaN planted in the host-side initial state is reported as an error
    status (no GPU fault: the value is uploaded as data)."""
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    m = small_model("surface")
    s = fw.Solver(m.ni, m.nj, m.nk, m.stept)
    inputs.attach(s, m)
    s.check()
    f = np.zeros(s.shape, np.float32)
    f[10, 10, 10] = np.nan
    s.set_field("Vx", f)
    with pytest.raises(fw.FwantError) as e:
        s.check()
    assert e.value.code == 4


def test_wait_deadline_reports_timeout(native_lib):
    """A bounded wait that runs out (a barrier phase nothing completes, 1000 polls) is
    reported as FWANT_ERR_TIMEOUT through the solver's device error word, and the solver
    then steps normally: the deadline path of the stage kernel, exercised without a fault."""
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    m = small_model("surface")
    s = inputs.attach(fw.Solver(m.ni, m.nj, m.nk, m.stept), m)
    with pytest.raises(fw.FwantError) as e:
        s.check_wait_timeout(1000)
    assert e.value.code == 5
    s.run(8)
    s.check()
    assert np.any(s.get_field("Vz"))


def test_set_media_rejects_nonpositive_rho(native_lib):
    """rho must be > 0 at every point, ghosts included (the solver divides by it); a zero
    or NaN anywhere is refused with INVALID_ARG before the medium on the device changes,
    and a valid medium is accepted afterwards."""
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    m = small_model("surface")
    s = fw.Solver(m.ni, m.nj, m.nk, m.stept)
    inputs.attach(s, m)
    for bad in (0.0, np.nan, -1.0):
        rho = m.rho.copy()
        rho[0, 5, 7] = bad  # a ghost point
        with pytest.raises(fw.FwantError) as e:
            s.set_media(m.lam, m.mu, rho)
        assert e.value.code == 1
    s.set_media(m.lam, m.mu, m.rho)
    s.run(8)
    s.check()


def test_interior_items_bitwise(oracle_mod, native_lib):
    """A grid with interior work items (tiles away from the PML, the sources and the free
    surface run the lean form of the stage kernel): still bit-identical to the oracle in
    the reference-order form, and both forms agree with it after a full 8-step cycle."""
    import fwant_gb300 as fw
    m = small_model("buried", ni=96, nj=40, nk=40)
    met = oracle_mod.metric(m.x, m.y, m.z)
    o = feed(oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface), m, met, "buried")
    ge = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept, exact_arith=True), m, met, "buried")
    gf = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept), m, met, "buried")
    for s in (ge, gf):
        s.planes_per_cta = 8  # chunks of 8 planes: interior chunks exist
    for s in (o, ge, gf):
        s.run(16)
    for c in range(9):
        b = interior(o.get_field(c))
        np.testing.assert_array_equal(interior(ge.get_field(c)), b.astype(np.float32))
        if np.any(b):
            assert rel_l2(interior(gf.get_field(c)), b) < 1e-5
