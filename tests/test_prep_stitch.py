"""`fwant_prep stitch`: a multi-rank input set (dims > 1, per-rank ni nj nk) read back as the
one-rank set of the same grid.  The per-rank files are cut from a one-rank set the way the
reference's preprocessors lay them out (tests/rank_split.py), with the ghost values a rank
holds for its neighbours poisoned; the stitched coord_, metric_ and media_ files equal the
one-rank files value for value, the sources (one of them inside several ranks' ghost
planes) come back once each, every receiver comes back with its global index, and the
written configuration names the stitched sizes, dims 1 1 1 and the new roots."""
import os
import subprocess

import numpy as np
import pytest

from rank_split import _read, split

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PREP = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_prep")
LENFD = 3


@pytest.mark.parametrize("dims", [(2, 2, 1), (3, 1, 2)])
def test_stitch_restores_the_one_rank_set(dims, tmp_path, native_lib):
    from fwant_gb300 import inputs
    n = (8, 10, 7)
    N = tuple(n[q] * dims[q] for q in range(3))
    m = inputs.make_model(*N, seed=4, npml=3, nrecv=12, source="buried", fc=2.0, t0=0.6)
    # a second force near the boundary between the first two ranks along x (inside both
    # ranks' ghost planes) and a third in the interior of the last rank
    ic = LENFD + n[0]
    extra = np.array([[ic, LENFD + 4, LENFD + 3], [LENFD + N[0] - 2, LENFD + N[1] - 3, LENFD + N[2] - 2]], np.int32)
    m.force_indx = np.concatenate([m.force_indx, extra]).astype(np.int32)
    m.force_shift = np.concatenate([m.force_shift, np.array([[0.1, -0.2, 0.3], [0.0, 0.0, -0.1]], np.float32)])
    m.force_t0 = np.concatenate([m.force_t0, np.array([0.5, 1.0], np.float32)])
    ntw = np.asarray(m.stf_time).size
    for attr, vals in (("fx", (1e14, 2e14)), ("fy", (0.0, -3e14)), ("fz", (5e14, 1e15))):
        a = np.asarray(getattr(m, attr), np.float32).reshape(-1, ntw)
        setattr(m, attr, np.concatenate([a, np.array(vals, np.float32)[:, None].repeat(ntw, 1)]))
    one = str(tmp_path / "one")
    inputs.write_inputs(m, one)
    ranks = str(tmp_path / "ranks")
    split(one, ranks, dims, n)
    conf = str(tmp_path / "SeisFD3D.conf")
    inputs.write_conf(conf, m, 16, {k: ranks for k in ("GRID_ROOT", "MEDIA_ROOT", "SOURCE_ROOT", "STATION_ROOT")}
                      | {"OUTPUT_ROOT": str(tmp_path / "out")})
    text = open(conf).read()
    for key, v in (("ni", n[0]), ("nj", n[1]), ("nk", n[2])):
        text = text.replace(f"{key} = {N['ijk'.index(key[1])]}", f"{key} = {v}")
    text = text.replace("dims = 1 1 1", "dims = %d %d %d" % dims)
    open(conf, "w").write(text)
    out = str(tmp_path / "stitched")
    os.makedirs(out)
    r = subprocess.run([PREP, "stitch", conf, "--out", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

    for name in ("coord", "metric", "media"):
        want, wdims, _ = _read(os.path.join(one, f"{name}_mpi000000.nc"))
        got, gdims, _ = _read(os.path.join(out, f"{name}_mpi000000.nc"))
        assert gdims == wdims
        for var, (a, vd, _) in want.items():
            assert got[var][1] == vd
            np.testing.assert_array_equal(got[var][0], a, err_msg=f"{name}:{var}")

    want, _, wat = _read(os.path.join(one, "source_mpi000000.nc"))
    got, _, gat = _read(os.path.join(out, "source_mpi000000.nc"))
    assert int(gat["number_of_force"]) == 3
    wrec = sorted(tuple(want["force_indx"][0][p]) + tuple(want["Fz"][0][p]) + tuple(want["force_shift"][0][p])
                  for p in range(3))
    grec = sorted(tuple(got["force_indx"][0][p]) + tuple(got["Fz"][0][p]) + tuple(got["force_shift"][0][p])
                  for p in range(3))
    assert wrec == grec
    np.testing.assert_array_equal(got["force_stf_time"][0], want["force_stf_time"][0])

    want, _, _ = _read(os.path.join(one, "station_mpi000000.nc"))
    got, _, _ = _read(os.path.join(out, "station_mpi000000.nc"))
    assert got["indx"][0].shape == want["indx"][0].shape
    key = lambda v: sorted(map(tuple, v))  # noqa: E731
    assert key(got["indx"][0]) == key(want["indx"][0])
    assert key(got["gindx"][0]) == key(want["gindx"][0])

    conf_out = open(os.path.join(out, "SeisFD3D.conf")).read()
    for key_, v in (("ni", N[0]), ("nj", N[1]), ("nk", N[2])):
        assert f"{key_} = {v}\n" in conf_out
    assert "dims = 1 1 1" in conf_out and f"GRID_ROOT = {out}" in conf_out and f"STATION_ROOT = {out}" in conf_out
