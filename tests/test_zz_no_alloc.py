"""fwant_get_snapshot_noalloc: snapshot extraction for callers that must not allocate
device memory (a GPU whose memory the wavefield fills, host programs with their own
allocator).  Its output must equal fwant_get_snapshot's on two calls in a row: the
second call, on a different sub-volume after more time steps, must not see anything left
in the shared fixed staging array by the first.  This file is collected last so that a
run stopping at the first failure has run every other test already."""
import numpy as np
import pytest

from helpers import feed, small_model

pytestmark = pytest.mark.gpu


def test_noalloc_snapshot_matches_allocating_entry_point(oracle_mod, native_lib):
    import fwant_gb300 as fw
    m = small_model("buried")
    met = oracle_mod.metric(m.x, m.y, m.z)
    s = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept), m, met, "buried")
    s.run(10)
    first = dict(subs=(4, 4, 4), subc=(m.ni, m.nj, m.nk), subt=(1, 1, 1),
                 comps=["Vx", "Vy", "Vz", "Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz"])
    a1 = s.get_snapshot_noalloc(**first)
    b1 = s.get_snapshot(**first)
    assert np.array_equal(a1, b1)
    assert np.any(a1)
    s.run(7)
    second = dict(subs=(6, 5, 7), subc=(5, 6, 4), subt=(3, 2, 2), comps=["Tzz", "Vx"])
    a2 = s.get_snapshot_noalloc(**second)
    b2 = s.get_snapshot(**second)
    assert np.array_equal(a2, b2)
    assert np.any(a2)
    assert a2.shape == (2, 5, 6, 4)


def test_noalloc_snapshot_rejects_requests_beyond_the_staging_size(native_lib):
    import fwant_gb300 as fw
    s = fw.Solver(160, 160, 40, 0.01)
    # 2 components x 160 x 160 x 40 = 2,048,000 values fit; 9 components (9,216,000) do not
    ok = s.get_snapshot_noalloc((4, 4, 4), (160, 160, 40), (1, 1, 1), comps=["Vx", "Vz"])
    assert ok.shape == (2, 160, 160, 40)
    with pytest.raises(fw.FwantError) as e:
        s.get_snapshot_noalloc((4, 4, 4), (160, 160, 40), (1, 1, 1), comps=list(range(9)))
    assert e.value.code == 1
    assert "staging" in str(e.value)
