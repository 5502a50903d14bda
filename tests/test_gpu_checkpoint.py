"""Checkpoint and resume: the complete state (wavefield, CFS-PML memory variables,
counters, records) is saved and restored, so a resumed run repeats the uninterrupted one
bit for bit; damaged files and files of another configuration are refused (the faults
are made on the host: truncated and altered files)."""
import os

import numpy as np
import pytest

from helpers import feed, small_model

pytestmark = pytest.mark.gpu


def _solver(oracle_mod, kind="nofree", **kw):
    import fwant_gb300 as fw
    m = small_model(kind, **kw)
    met = oracle_mod.metric(m.x, m.y, m.z)
    s = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface), m, met, kind)
    s.set_sgt_record((5, 5, 5), (5, 4, 3), (3, 3, 3), 3, 40)
    return s


@pytest.mark.parametrize("kind", ["nofree", "surface"])
def test_resume_repeats_the_uninterrupted_run(kind, oracle_mod, native_lib, tmp_path):
    path = os.path.join(tmp_path, "state.ckpt")
    a = _solver(oracle_mod, kind)
    a.run(21)   # mid-cycle (21 = 2 blocks + 5)
    a.save_checkpoint(path)
    a.run(27)
    b = _solver(oracle_mod, kind)
    b.load_checkpoint(path)
    assert b.ntime == 21
    b.run(27)
    for c in range(9):
        np.testing.assert_array_equal(a.get_field(c), b.get_field(c))
    np.testing.assert_array_equal(a.get_seismo(), b.get_seismo())
    np.testing.assert_array_equal(a.get_sgt(), b.get_sgt())


def test_damaged_or_foreign_files_are_refused(oracle_mod, native_lib, tmp_path):
    import fwant_gb300 as fw
    path = os.path.join(tmp_path, "state.ckpt")
    a = _solver(oracle_mod)
    a.run(5)
    a.save_checkpoint(path)
    raw = open(path, "rb").read()
    b = _solver(oracle_mod)
    for name, data in (("truncated", raw[:-100]), ("altered", raw[:-10] + bytes([raw[-10] ^ 1]) + raw[-9:]),
                       ("garbage", b"not a checkpoint" * 100)):
        bad = os.path.join(tmp_path, name)
        open(bad, "wb").write(data)
        with pytest.raises(fw.FwantError) as e:
            b.load_checkpoint(bad)
        assert e.value.code == 1, name
    with pytest.raises(fw.FwantError) as e:
        b.load_checkpoint(os.path.join(tmp_path, "missing"))
    assert e.value.code == 1
    other = _solver(oracle_mod, ni=30)
    with pytest.raises(fw.FwantError) as e:
        other.load_checkpoint(path)
    assert e.value.code == 6
    # the refused loads left b untouched: it still runs from its own initial state
    assert b.ntime == 0
    b.load_checkpoint(path)
    assert b.ntime == 5
