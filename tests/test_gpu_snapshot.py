"""Snapshot extraction (io_wave_export) against the full field and the oracle."""
import numpy as np
import pytest

from helpers import feed, small_model

pytestmark = pytest.mark.gpu


def test_snapshot_matches_full_field_and_oracle(oracle_mod, native_lib):
    import fwant_gb300 as fw
    m = small_model("buried")
    met = oracle_mod.metric(m.x, m.y, m.z)
    g = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept, exact_arith=True), m, met, "buried")
    o = feed(oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept), m, met, "buried")
    g.run(12)
    o.run(12)
    subs, subc, subt = (5, 4, 6), (7, 5, 4), (3, 2, 3)
    comps = ["Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz", "Vz"]
    snap = g.get_snapshot(subs, subc, subt, comps)
    assert snap.shape == (len(comps), 7, 5, 4)
    for n, c in enumerate(comps):
        full = g.get_field(c)
        ref = o.get_field(c)
        sl = tuple(slice(s - 1, s - 1 + t * (k - 1) + 1, t) for s, k, t in zip(subs, subc, subt))
        assert np.array_equal(snap[n], full[sl])
        assert np.array_equal(snap[n], ref[sl].astype(np.float32))


def test_snapshot_rejects_bad_requests(native_lib):
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    m = small_model("surface")
    s = inputs.attach(fw.Solver(m.ni, m.nj, m.nk, m.stept), m)
    with pytest.raises(fw.FwantError):
        s.get_snapshot((1, 4, 4), (2, 2, 2), (1, 1, 1))  # starts in the ghost layer
    with pytest.raises(fw.FwantError):
        s.get_snapshot((4, 4, 4), (m.ni + 1, 1, 1), (1, 1, 1))  # runs past the interior
    with pytest.raises(fw.FwantError):
        s.get_snapshot((4, 4, 4), (2, 2, 2), (0, 1, 1))  # zero stride
    # stride x (count - 1) = 2^32 wraps a 32-bit end index back to the start: every entry
    # point that takes a sub-volume refuses it on the host, before any launch
    wrap = dict(subs=(4, 4, 4), subc=(65537, 1, 1), subt=(65536, 1, 1))
    for call in (lambda: s.get_snapshot(**wrap), lambda: s.get_snapshot_noalloc(**wrap),
                 lambda: s.set_sgt_record(wrap["subs"], wrap["subc"], wrap["subt"], 1, 4)):
        with pytest.raises(fw.FwantError) as e:
            call()
        assert e.value.code == 1
