"""Batched launch: uneven simulations stepped together give the results of running each
one alone.  The reference-order form (no contraction) agrees bit for bit; in the fast form
the compiler contracts multiply-adds separately in the batched and the single-simulation
kernels, so the two agree to FP32 rounding (relative L2 below 1e-6 after 40 steps)."""
import numpy as np
import pytest

from helpers import feed, rel_l2, small_model

pytestmark = pytest.mark.gpu

MEMBERS = [("surface", (26, 22, 20)), ("buried", (40, 33, 25)), ("nofree", (17, 30, 18)), ("moment", (33, 19, 27))]


def _members(oracle_mod, exact, seed=3):
    import fwant_gb300 as fw
    out = []
    for kind, (ni, nj, nk) in MEMBERS:
        m = small_model(kind, ni=ni, nj=nj, nk=nk, seed=seed)
        met = oracle_mod.metric(m.x, m.y, m.z)
        make = lambda: feed(fw.Solver(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface, exact_arith=exact),
                            m, met, kind)
        out.append((make(), make()))
    return out


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_batch_equals_single_runs(exact, oracle_mod, native_lib):
    import fwant_gb300 as fw
    pairs = _members(oracle_mod, exact)
    batched = [p[0] for p in pairs]
    alone = [p[1] for p in pairs]
    b = fw.Batch(batched)
    b.run(3)    # eager steps up to ...
    b.run(21)   # ... a graph block boundary, then graph blocks and an eager remainder
    b.run(16)
    for s in alone:
        s.run(40)
    def same(x, y):
        if exact:
            np.testing.assert_array_equal(x, y)
        elif np.any(y):
            assert rel_l2(x, y) < 1e-6

    for sb, sa in zip(batched, alone):
        assert sb.ntime == sa.ntime == 40
        for c in range(9):
            same(sb.get_field(c), sa.get_field(c))
        # seismograms by group: on the free surface Tzz, Txz and Tyz are rounding noise
        gb, ga = sb.get_seismo(), sa.get_seismo()
        same(gb[:3], ga[:3])
        same(gb[3:], ga[3:])
    # members stay usable on their own after batch runs
    batched[1].run(5)
    alone[1].run(5)
    same(batched[1].get_field("Vz"), alone[1].get_field("Vz"))


@pytest.mark.parametrize("ctas", [1, 7, 152, 10000])
def test_batch_any_grid_size(ctas, oracle_mod, native_lib):
    """The persistent grid may be smaller or larger than the number of work items."""
    import fwant_gb300 as fw
    pairs = _members(oracle_mod, True)[:2]
    b = fw.Batch([p[0] for p in pairs])
    b.set_ctas(ctas)
    b.run(9)
    for s, ref in pairs:
        ref.run(9)
        for c in (0, 2, 5):
            np.testing.assert_array_equal(s.get_field(c), ref.get_field(c))


def test_batch_with_sgt_record_and_planes(oracle_mod, native_lib):
    import fwant_gb300 as fw
    pairs = _members(oracle_mod, True)[:3]
    for s, ref in pairs:
        for x in (s, ref):
            x.set_sgt_record((5, 5, 5), (6, 5, 4), (2, 2, 3), 2, 8)
    pairs[0][0].planes_per_cta = 5   # members with different k-chunks
    pairs[2][0].planes_per_cta = 64
    b = fw.Batch([p[0] for p in pairs])
    b.run(16)
    for s, ref in pairs:
        ref.run(16)
        np.testing.assert_array_equal(s.get_sgt(), ref.get_sgt())
        np.testing.assert_array_equal(s.get_field("Txx"), ref.get_field("Txx"))


def test_batch_rules(oracle_mod, native_lib):
    import fwant_gb300 as fw
    pairs = _members(oracle_mod, True)[:2]
    a, b = pairs[0][0], pairs[1][0]
    with pytest.raises(fw.FwantError):
        fw.Batch([a, a])
    a.run(1)
    bt = fw.Batch([a, b])
    with pytest.raises(fw.FwantError) as e:
        bt.run(4)   # not at the same time step
    assert e.value.code == 6
    m = small_model("surface")
    c = fw.Solver(m.ni, m.nj, m.nk, m.stept, exact_arith=False)
    with pytest.raises(fw.FwantError):
        fw.Batch([b, c])   # different arithmetic form


def test_autotune_keeps_results(oracle_mod, native_lib):
    """Tuning runs trial steps and restores the initial state: a tuned solver then gives
    the results of an untuned one bit for bit (planes per CTA only move work between
    CTAs), and a tuned batch those of its members run alone."""
    import fwant_gb300 as fw
    pairs = _members(oracle_mod, False)[:3]
    tuned, plain = pairs[0]
    kc = tuned.autotune(2)
    assert kc >= 3 and tuned.ntime == 0 and tuned.planes_per_cta == kc
    for s in (tuned, plain):
        s.run(20)
    for c in range(9):
        np.testing.assert_array_equal(tuned.get_field(c), plain.get_field(c))
    np.testing.assert_array_equal(tuned.get_seismo(), plain.get_seismo())
    members = [p[0] for p in pairs[1:]]
    alone = [p[1] for p in pairs[1:]]
    b = fw.Batch(members)
    ctas = b.autotune(2)
    assert ctas >= 0 and all(m.ntime == 0 for m in members)
    b.run(12)
    for m, a in zip(members, alone):
        a.run(12)
        assert rel_l2(m.get_field("Vz"), a.get_field("Vz")) < 1e-6
    with pytest.raises(fw.FwantError) as e:
        tuned.autotune(2)   # after the first step
    assert e.value.code == 6


def test_lean_stage_split_keeps_results(oracle_mod, native_lib):
    """Running every stage as one full launch (lean stages 0), or splitting every stage
    into interior-only and full launches (7), instead of splitting stages 1 and 4 (the
    default 5) moves work between kernels only: the same fields bit for bit in the
    reference-order form.  Masks beyond the three stage bits are refused."""
    import fwant_gb300 as fw
    (one, split), (three, ref3) = _members(oracle_mod, True)[:2]
    assert split.lean_stages == 5
    one.lean_stages = 0
    three.lean_stages = 7
    for s in (one, split, three, ref3):
        s.run(16)
    for c in range(9):
        np.testing.assert_array_equal(one.get_field(c), split.get_field(c))
        np.testing.assert_array_equal(three.get_field(c), ref3.get_field(c))
    with pytest.raises(fw.FwantError):
        one.lean_stages = 8
