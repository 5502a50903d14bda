"""The preprocessing chain on the GPU, all from configuration files: fwant_prep grid,
metric, source and station, fwant_media, then fwant_wave, as the reference runs
seis3d_grid, seis3d_metric, seis3d_source, seis3d_station, seis3d_media and the solver.
The metric stage writes the values of the solver's own fwant_compute_metric bit for bit,
and the solver stage run on the chain's files records the seismograms of the same solve
through the library API fed from the arrays in those files."""
import os
import subprocess

import numpy as np
import pytest

import prep_case as pc

pytestmark = pytest.mark.gpu

WAVE = os.path.join(pc.ROOT, "fwant_gb300", "bin", "fwant_wave")
MEDIA = os.path.join(pc.ROOT, "fwant_gb300", "bin", "fwant_media")
NI, NJ, NK = 28, 24, 18


def test_metric_stage_equals_the_solver(native_lib, tmp_path):
    import fwant_gb300 as fw
    tmp = str(tmp_path)
    rng = np.random.default_rng(2)
    z = (np.float32(6371.0) - np.cumsum(rng.uniform(0.4, 1.5, NK))[::-1]).astype(np.float32)
    pc.grid_conf(tmp, steph=(0.009, 0.0075, 0.0), lists=[("<z", z)])
    conf = pc.main_conf(tmp, ni=NI, nj=NJ, nk=NK)
    pc.run("grid", conf)
    pc.run("metric", conf)
    c, _, _ = pc.read(os.path.join(tmp, "coord_mpi000000.nc"))
    got, _, dims = pc.read(os.path.join(tmp, "metric_mpi000000.nc"))
    assert dims == {"I": NI + 6, "J": NJ + 6, "K": NK + 6}
    s = fw.Solver(NI, NJ, NK, 0.01)
    s.set_coord(c["x"], c["y"], c["z"])
    s.compute_metric()
    want = s.get_metric()
    alone = fw.metric(c["x"], c["y"], c["z"])
    assert set(got) == set(want) == set(alone)
    for k in want:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
        np.testing.assert_array_equal(alone[k], want[k], err_msg=k)


def _deg(a):
    return float(np.degrees(np.float64(a)))


def test_chain_into_the_solver(native_lib, tmp_path):
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    tmp = str(tmp_path)
    out = os.path.join(tmp, "out")
    os.makedirs(out)
    pc.grid_conf(tmp)
    pc.run("grid", pc.main_conf(tmp, ni=NI, nj=NJ, nk=NK))
    c, _, _ = pc.read(os.path.join(tmp, "coord_mpi000000.nc"))
    x, y, z = c["x"], c["y"], c["z"]

    model = os.path.join(tmp, "cart1d.dat")
    inputs.write_cart1d_file(model, [0.0, 2000.0, 4000.0, 1.0e5], [2400.0, 2600.0, 2800.0, 3300.0],
                             [5000.0, 5500.0, 6000.0, 8000.0], [2900.0, 3200.0, 3450.0, 4600.0])
    inputs.write_media_conf(os.path.join(tmp, "SeisMedia.conf"), ("cart1d", "ascii", model))
    pc.source_conf(tmp, 6370000.0,
                   [(_deg(x[14]) + 0.002, _deg(y[12]), 6.5e6, 0.0, 1.0e15, 0.0, 0.3, 1.0)], 1,
                   [(_deg(x[12]), _deg(y[10]) + 0.003, 6371000.0 - 4200.0, 0.0, 1.0e15, 30.0, 60.0, 90.0)], 1,
                   "angle")
    extra = [f"MEDIA_CONF = {tmp}/SeisMedia.conf", f"MEDIA_ROOT = {tmp}", f"OUTPUT_ROOT = {out}",
             "abs_number = 5 5 5 5 5 0", "abs_velocity = 6000.0 6000.0 6000.0 6000.0 6000.0 6000.0",
             "CFS_bmax = 2.0 2.0 2.0 2.0 2.0 2.0", "CFS_amax = 0.5 0.5 0.5 0.5 0.5 0.5", "number_of_snap = 0",
             "number_of_recv = 3", "number_of_inline = 1", "tinv_of_seismo = 1", "topo_hyper_height = 6371000.0",
             f"recv_001 = {_deg(x[16])} {_deg(y[15])} 6.4e6",
             f"recv_002 = {_deg(x[10]) + 0.001} {_deg(y[9])} 6369000.0",
             f"recv_003 = {_deg(x[18])} {_deg(y[8]) - 0.002} 6371000.0",
             f"line_001 = {_deg(x[9])} {_deg(y[14])} 6.4e6 0.009 0.0 0.0 8"]
    conf = pc.main_conf(tmp, extra, ni=NI, nj=NJ, nk=NK)
    for stage in ("metric", "source", "station"):
        pc.run(stage, conf)
    r = subprocess.run([MEDIA, conf], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    dtmax = float(r.stdout.split("Maximum allowed time step is")[1].split()[0])
    assert dtmax > 0.01
    r = subprocess.run([WAVE, conf], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

    # the same solve through the library, fed from the chain's files
    met, _, _ = pc.read(os.path.join(tmp, "metric_mpi000000.nc"))
    med, _, _ = pc.read(os.path.join(tmp, "media_mpi000000.nc"))
    src, satt, _ = pc.read(os.path.join(tmp, "source_mpi000000.nc"))
    sta, tatt, _ = pc.read(os.path.join(tmp, "station_mpi000000.nc"))
    assert sta["indx"].shape == (11, 3)
    s = fw.Solver(NI, NJ, NK, 0.01)
    s.set_coord(x, y, z)
    s.set_metric(met["xsin"], met["xcot"], met["xi_x"], met["eta_y"], met["zeta_z"])
    s.set_media(*(med[k].transpose(2, 1, 0) for k in ("lambda", "mu", "rho")))
    s.set_pml([5, 5, 5, 5, 5, 0], [6000.0] * 6, [2.0] * 6, [0.5] * 6)
    s.set_forces(src["force_indx"], src["force_shift"], src["force_start_time"], src["force_stf_time"],
                 src["force_stf_freq"], src["Fx"], src["Fy"], src["Fz"], int(satt["force_stf_id"]))
    s.set_moments(src["moment_indx"], src["moment_shift"], src["moment_start_time"], src["moment_stf_time"],
                  src["moment_stf_freq"], np.stack([src[k] for k in ("Mxx", "Myy", "Mzz", "Mxy", "Mxz", "Myz")]),
                  int(satt["moment_stf_id"]))
    s.set_receivers(sta["indx"], int(tatt["tinv"]))
    total = fw.reference_steps(10)
    s.run(total)
    seis, _, _ = pc.read(os.path.join(out, "seismo_mpi000000.nc"))
    api = s.get_seismo()
    for ci, name in enumerate(fw.COMPONENTS):
        assert seis[name].shape == (total, 11)
        np.testing.assert_array_equal(seis[name], api[ci], err_msg=name)
    assert np.all(np.isfinite(api)) and np.any(api[2] != 0.0)
