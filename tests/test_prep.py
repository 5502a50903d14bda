"""fwant_prep, the input preprocessors as one program (the reference's seis3d_grid,
seis3d_source and seis3d_station on one rank): configuration files in, the coord_, source_
and station_ NetCDF files out, equal bit for bit to the CPU restatement in
oracle/prep_oracle.py.  These stages run on the host, so they are tested without a GPU; the
metric stage and the whole chain into the solver are in tests/test_gpu_fwant_prep.py."""
import os
import subprocess

import numpy as np
import pytest

from prep_case import EXE, NI, NJ, NK, f32text, grid_conf, main_conf, read, run, source_conf, write


@pytest.fixture
def grid_dir(tmp_path, native_lib):
    tmp = str(tmp_path)
    grid_conf(tmp)
    run("grid", main_conf(tmp))
    return tmp


def test_grid_uniform_axes(grid_dir):
    from oracle import prep_oracle as P

    from fwant_gb300 import inputs
    v, _, dims = read(os.path.join(grid_dir, "coord_mpi000000.nc"))
    assert dims == {"I": NI + 6, "J": NJ + 6, "K": NK + 6}
    want = {"x": P.grid_axis(NI, 0.009, 45.5), "y": P.grid_axis(NJ, 0.009, 100.0),
            "z": P.grid_axis(NK, 0.5, 6371.0, top=True, degrees=False, d2m=1000.0)}
    for k in "xyz":
        np.testing.assert_array_equal(v[k], want[k], err_msg=k)
    # the library's own generator of the same axes agrees
    np.testing.assert_array_equal(v["x"], inputs.grid_coords(NI, 0.009, 45.5, None, 1.0, degrees=True))
    np.testing.assert_array_equal(v["z"], inputs.grid_coords(NK, 0.5, 6371.0, None, 1000.0, degrees=False,
                                                             top_anchored=True))
    # the free surface sits at rmax
    assert v["z"][3 + NK - 1] == np.float32(6371000.0)


def test_grid_listed_axes(tmp_path, native_lib):
    from oracle import prep_oracle as P
    tmp = str(tmp_path)
    rng = np.random.default_rng(4)
    y = np.cumsum(rng.uniform(0.005, 0.012, NJ)).astype(np.float32) + np.float32(99.0)
    z = (np.float32(6371.0) - np.cumsum(rng.uniform(0.4, 2.0, NK))[::-1]).astype(np.float32)
    grid_conf(tmp, steph=(0.009, 0.0, 0.0), lists=[("<y", y), ("<z", z)])
    run("grid", main_conf(tmp))
    v, _, _ = read(os.path.join(tmp, "coord_mpi000000.nc"))
    np.testing.assert_array_equal(v["x"], P.grid_axis(NI, 0.009, 45.5))
    np.testing.assert_array_equal(v["y"], P.grid_axis(NJ, 0.0, 0.0, values=y))
    np.testing.assert_array_equal(v["z"], P.grid_axis(NK, 0.0, 0.0, values=z, degrees=False, d2m=1000.0))
    # a list shorter than the axis stops the program with a message
    grid_conf(tmp, steph=(0.009, 0.0, 0.0), lists=[("<y", y[:-3]), ("<z", z)])
    r = run("grid", main_conf(tmp), ok=False)
    assert r.returncode != 0 and "not a number: <z" in r.stderr


def _coords(tmp):
    v, _, _ = read(os.path.join(tmp, "coord_mpi000000.nc"))
    return v["x"], v["y"], v["z"]


def test_station_locating(grid_dir):
    from oracle import prep_oracle as P
    tmp = grid_dir
    x, y, z = _coords(tmp)
    deg = lambda a: float(np.degrees(np.float64(a)))
    thh = 6371000.0
    recvs = [(deg(x[8]) + 0.0021, deg(y[7]) - 0.003, 6371000.0 - 2300.0),   # buried: nearest node in depth
             (deg(x[10]), deg(y[12]) + 0.004, 6.4e6),                      # above the surface height: k = nk2
             (deg(x[3]) - 0.02, deg(y[9]), 6371000.0),                     # nearest node a ghost: dropped
             (deg(x[12]) + 0.001, deg(y[5]), 6371000.0 - 5600.0)]          # just below the bottom node
    lines = [(deg(x[5]), deg(y[4]), 6.4e6, 0.009, 0.0045, 0.0, 6),
             (deg(x[15]), deg(y[10]), 6371000.0 - 500.0, 0.0, 0.0, -700.0, 5)]
    extra = [f"number_of_recv = {len(recvs)}", f"number_of_inline = {len(lines)}", "tinv_of_seismo = 3",
             f"topo_hyper_height = {f32text(thh)}"]
    extra += [f"recv_{n:03d} = " + " ".join(f32text(v) for v in r) for n, r in enumerate(recvs, start=1)]
    extra += [f"line_{n:03d} = " + " ".join(f32text(v) for v in ln[:6]) + f" {ln[6]}" for n, ln in enumerate(lines, start=1)]
    conf = main_conf(tmp, extra)
    run("station", conf)
    v, att, dims = read(os.path.join(tmp, "station_mpi000000.nc"))
    xyz, ids = P.station_points(recvs, lines)
    want = P.receiver_locate(xyz, ids, x, y, z, NI, NJ, NK, thh)
    assert len(want["indx"]) == len(recvs) + sum(ln[6] for ln in lines) - 1
    for k in ("indx", "gindx", "coord", "grid", "id"):
        np.testing.assert_array_equal(v[k], want[k], err_msg=k)
    assert int(att["tinv"]) == 3 and dims["num_pt"] is None
    assert v["indx"][1, 2] == NK + 3 and v["indx"][2, 2] == 4   # the surface point; the bottom node


def _check_sources(v, att, kind, comps, axis, t0, vals, x, y, z, hyper, stf_id, stf_name):
    from oracle import prep_oracle as P
    indx, axis2, shift, found = P.locate_sources(axis, x, y, z, NI, NJ, NK, hyper)
    assert found.all()
    np.testing.assert_array_equal(v[f"{kind}_indx"], indx)
    np.testing.assert_array_equal(v[f"{kind}_axis"], axis2)
    np.testing.assert_array_equal(v[f"{kind}_shift"], shift)
    np.testing.assert_array_equal(v[f"{kind}_start_time"], t0)
    for c, name in enumerate(comps):
        np.testing.assert_array_equal(v[name], vals[c], err_msg=name)
    assert int(att[f"{kind}_stf_id"]) == stf_id
    assert att[f"{kind}_stf_type"].decode() == stf_name
    return indx, shift


def test_source_forces_and_angle_moments(grid_dir):
    from oracle import prep_oracle as P
    tmp = grid_dir
    x, y, z = _coords(tmp)
    deg = lambda a: float(np.degrees(np.float64(a)))
    hyper = 6370000.0
    ntw_f, ntw_m = 2, 1
    fr = [(deg(x[9]) + 0.003, deg(y[8]) - 0.002, 6.5e6, 0.5, 1.0e15, 0.0, 0.25, 1.0),   # above: surface node
          (deg(x[9]) + 0.003, deg(y[8]) - 0.002, 6.5e6, 0.5, 2.0e15, 1.0, 0.0, -0.5),
          (deg(x[11]) - 0.0025, deg(y[6]) + 0.001, 6371000.0 - 1700.0, 1.25, 3.0e14, 0.3, 0.6, 0.9),
          (deg(x[11]) - 0.0025, deg(y[6]) + 0.001, 6371000.0 - 1700.0, 1.25, 3.0e14, 0.7, -0.2, 0.1)]
    mo = [(deg(x[7]), deg(y[7]) + 0.0031, 6371000.0 - 3100.0, 0.0, 1.0e16, 30.0, 60.0, 90.0),
          (deg(x[13]) + 0.001, deg(y[9]), 6371000.0 - 900.0, 0.2, 5.0e15, 217.5, 33.3, -41.0)]
    source_conf(tmp, hyper, fr, ntw_f, mo, ntw_m, "angle")
    run("source", main_conf(tmp))
    v, att, dims = read(os.path.join(tmp, "source_mpi000000.nc"))
    assert int(att["number_of_force"]) == 2 and int(att["number_of_moment"]) == 2
    assert dims["force_time_window"] == ntw_f and dims["moment_point"] == 2
    axis, t0, F = P.forces(fr, ntw_f)
    indx, shift = _check_sources(v, att, "force", ("Fx", "Fy", "Fz"), axis, t0, F, x, y, z, hyper, 200, "ricker")
    assert indx[0, 2] == NK + 3 and shift[0, 2] == 0.0 and v["force_axis"][0, 2] == z[NK + 2]
    assert np.all(np.abs(shift[1]) < 1.0) and np.any(shift[1] != 0.0)
    np.testing.assert_array_equal(v["force_stf_time"], np.float32([1.5, 2.5]))
    axis, t0, M = P.moments(mo, ntw_m, "angle")
    _check_sources(v, att, "moment", ("Mxx", "Myy", "Mzz", "Mxy", "Mxz", "Myz"), axis, t0, M, x, y, z, hyper,
                   220, "gauss")
    # a double couple is trace-free
    assert abs(float(M[0, 0, 0] + M[1, 0, 0] + M[2, 0, 0])) <= 1e-6 * abs(float(M[2, 0, 0]))


def test_source_moment_tensors_and_errors(grid_dir):
    from oracle import prep_oracle as P
    tmp = grid_dir
    x, y, z = _coords(tmp)
    deg = lambda a: float(np.degrees(np.float64(a)))
    hyper = 6370000.0
    mo = [(deg(x[8]), deg(y[8]), 6371000.0 - 2000.0, 0.1, 1.0e15, 1.0, -0.5, -0.5, 0.2, 0.1, 0.3),
          (deg(x[8]), deg(y[8]), 6371000.0 - 2000.0, 0.1, 1.0e15, 0.5, 0.5, -1.0, 0.0, 0.0, 0.0)]
    source_conf(tmp, hyper, [], 0, mo, 2, "moment", stf_m="bell_int")
    run("source", main_conf(tmp))
    v, att, _ = read(os.path.join(tmp, "source_mpi000000.nc"))
    assert int(att["number_of_force"]) == 0 and "Fx" not in v
    axis, t0, M = P.moments(mo, 2, "moment")
    _check_sources(v, att, "moment", ("Mxx", "Myy", "Mzz", "Mxy", "Mxz", "Myz"), axis, t0, M, x, y, z, hyper,
                   100, "bell_int")
    # a buried source below the surface-height limit outside the grid: the reference stops
    out = [(deg(x[8]), deg(y[8]), 6.0e6, 0.0, 1.0e15, 0.0, 0.0, 1.0)]
    source_conf(tmp, hyper, out, 1, [], 0, "angle")
    r = run("source", main_conf(tmp), ok=False)
    assert r.returncode == 1 and "out of the computational domain" in r.stdout
    # an STF name the reference does not know
    source_conf(tmp, hyper, [(deg(x[8]), deg(y[8]), 6.5e6, 0.0, 1.0, 0.0, 0.0, 1.0)], 1, [], 0, "angle",
                 stf_f="boxcar")
    r = run("source", main_conf(tmp), ok=False)
    assert r.returncode != 0 and "Have you told me how to generate the STF of boxcar" in r.stderr


def test_prep_rejects_bad_setups(grid_dir):
    r = subprocess.run([EXE, "mesh", main_conf(grid_dir)], capture_output=True, text=True)
    assert r.returncode != 0 and "unknown stage" in r.stderr
    conf = main_conf(grid_dir, ["dims = 2 1 1"])
    # dims is read from the first line that has the key: the earlier "dims = 1 1 1" wins
    assert run("grid", conf).returncode == 0
    path = os.path.join(grid_dir, "bad.conf")
    write(path, ["ni = 20", "nj = 16", "nk = 12", "dims = 1 2 1", f"GRID_CONF = {grid_dir}/SeisGrid.conf",
                  f"GRID_ROOT = {grid_dir}"])
    r = run("grid", path, ok=False)
    assert r.returncode != 0 and "dims must be 1 1 1" in r.stderr


def test_angle2moment_known_answers(grid_dir):
    """Aki & Richards' double couples: a vertical strike-slip fault striking north has only
    M12 = M0 (Mxy = -M0 in theta, phi, r); a thrust on a 45-degree plane striking north has
    M22 = -M0 and M33 = +M0.  Checked on the restatement and through the program's file."""
    from oracle import prep_oracle as P
    tiny = 1e-12
    ss = P.angle2moment(0.0, 90.0, 0.0)
    assert float(ss[3]) == -1.0 and all(abs(float(ss[c])) < tiny for c in (0, 1, 2, 4, 5))
    th = P.angle2moment(0.0, 45.0, 90.0)
    assert float(th[1]) == -1.0 and float(th[2]) == 1.0
    assert all(abs(float(th[c])) < tiny for c in (0, 3, 4, 5))
    x, y, z = _coords(grid_dir)
    deg = lambda a: float(np.degrees(np.float64(a)))
    mo = [(deg(x[8]), deg(y[8]), 6371000.0 - 2000.0, 0.0, 2.0, 0.0, 90.0, 0.0),
          (deg(x[9]), deg(y[9]), 6371000.0 - 2000.0, 0.0, 3.0, 0.0, 45.0, 90.0)]
    source_conf(grid_dir, 6370000.0, [], 0, mo, 1, "angle")
    run("source", main_conf(grid_dir))
    v, _, _ = read(os.path.join(grid_dir, "source_mpi000000.nc"))
    assert v["Mxy"][0, 0] == -2.0 and v["Myy"][1, 0] == -3.0 and v["Mzz"][1, 0] == 3.0
