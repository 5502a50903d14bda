"""`fwant_wave`, the solver stage as a program: SeisFD3D.conf and the reference's NetCDF
input files in, seismo_ and vel_/sgt_ snapshot files out.  Its outputs equal the same
solve through the library API bit for bit, and a run resumed from a checkpoint writes the
files of the uninterrupted run."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import small_model

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_wave")
NT = 30  # the reference runs 32 steps (whole 8-step blocks)
SNAPS = [((-1, -1, -2), (-1, -1, 1), (2, 2, 1), 4, 3, "V"),    # surface velocity every 4 steps
         ((3, 4, 5), (5, 4, 3), (2, 3, 2), 8, 2, "TV")]         # a sub-volume, stress and velocity


def _prepare(tmp, **conf):
    from fwant_gb300 import inputs
    m = small_model("surface")
    inputs.write_inputs(m, tmp)
    roots = {k: tmp for k in ("GRID_ROOT", "MEDIA_ROOT", "SOURCE_ROOT", "STATION_ROOT")}
    roots["OUTPUT_ROOT"] = os.path.join(tmp, "out")
    roots["CHECKPOINT_ROOT"] = os.path.join(tmp, "ckpt")
    os.makedirs(roots["OUTPUT_ROOT"], exist_ok=True)
    os.makedirs(roots["CHECKPOINT_ROOT"], exist_ok=True)
    path = os.path.join(tmp, "SeisFD3D.conf")
    inputs.write_conf(path, m, NT, roots, snaps=SNAPS, **conf)
    return m, path, roots


def _run(conf):
    r = subprocess.run([EXE, conf], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r


def _read(path):
    from scipy.io import netcdf_file
    with netcdf_file(path, "r", mmap=False) as f:
        return {k: np.array(v[:]) for k, v in f.variables.items()}, dict(f._attributes)


def _keep_records(path, n):
    """Rewrite a snapshot file with its first n records."""
    from scipy.io import netcdf_file
    with netcdf_file(path, "r", mmap=False) as f:
        dims = dict(f.dimensions)
        att = dict(f._attributes)
        data = {k: (v.typecode(), v.dimensions, np.array(v[:])) for k, v in f.variables.items()}
    with netcdf_file(path, "w", version=1) as g:
        g.createDimension("time", None)
        for d, ln in dims.items():
            if ln is not None:
                g.createDimension(d, ln)
        for k, a in att.items():
            setattr(g, k, a)
        for k, (tc, dm, a) in data.items():
            v = g.createVariable(k, tc, dm)
            v[:n] = a[:n]


def test_outputs_equal_the_library_solve(native_lib, tmp_path):
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    tmp = str(tmp_path)
    m, conf, roots = _prepare(tmp)
    _run(conf)
    out = roots["OUTPUT_ROOT"]
    # the same solve through the API, snapshots taken at the same steps
    s = inputs.attach(fw.Solver(m.ni, m.nj, m.nk, m.stept), m, metric=inputs.metric_fp64(m.x, m.y, m.z))
    total = fw.reference_steps(NT)
    frames = {1: [], 2: []}
    for step in range(1, total + 1):
        s.run(1)
        if step % 4 == 0:
            frames[1].append(s.get_snapshot((4, 4, 3 + m.nk), (m.ni // 2 + m.ni % 2, m.nj // 2 + m.nj % 2, 1),
                                            (2, 2, 1), comps=("Vx", "Vy", "Vz")))
        if step % 8 == 0:
            frames[2].append(s.get_snapshot((6, 7, 8), (5, 4, 3), (2, 3, 2),
                                            comps=("Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz", "Vx", "Vy", "Vz")))
    seis, att = _read(os.path.join(out, "seismo_mpi000000.nc"))
    api = s.get_seismo()
    assert att["title"] == b"seismograms"
    assert seis["Vx"].shape == (total, m.recv_indx.shape[0])
    for c, name in enumerate(fw.COMPONENTS):
        np.testing.assert_array_equal(seis[name], api[c])
    np.testing.assert_allclose(seis["time"], np.float32(m.stept) * np.arange(1, total + 1, dtype=np.float32),
                               rtol=1e-6)
    # surface velocity: files of 3 frames (steps 4-12, 16-24, 28-32)
    got = []
    for n in (1, 2, 3):
        v, a = _read(os.path.join(out, f"vel_001_mpi000000_n{n:05d}.nc"))
        assert list(a["subt"]) == [2, 2, 1] and list(a["gsubs"]) == [1, 1, m.nk]
        got.append(np.stack([v["Vx"], v["Vy"], v["Vz"]], axis=1))   # (t, c, K, J, I)
    got = np.concatenate(got)
    want = np.stack(frames[1]).transpose(0, 1, 4, 3, 2)            # (t, c, i, j, k) -> (t, c, K, J, I)
    np.testing.assert_array_equal(got, want)
    # sub-volume: stress file and velocity file, 2 frames each (steps 8-16, 24-32)
    for n in (1, 2):
        t, _ = _read(os.path.join(out, f"sgt_002_mpi000000_n{n:05d}.nc"))
        v, _ = _read(os.path.join(out, f"vel_002_mpi000000_n{n:05d}.nc"))
        for f in range(2):
            w = frames[2][2 * (n - 1) + f].transpose(0, 3, 2, 1)
            for c, name in enumerate(("Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz")):
                np.testing.assert_array_equal(t[name][f], w[c])
            for c, name in enumerate(("Vx", "Vy", "Vz")):
                np.testing.assert_array_equal(v[name][f], w[6 + c])


def test_resume_writes_the_uninterrupted_files(native_lib, tmp_path):
    full = os.path.join(str(tmp_path), "full")
    part = os.path.join(str(tmp_path), "part")
    os.makedirs(full)
    os.makedirs(part)
    _, conf_full, roots_full = _prepare(full)
    _run(conf_full)
    # the interrupted run: checkpoints every 12 steps (12, 24; the last one kept)...
    _, conf_part, roots_part = _prepare(part, checkpoint_tinv=12)
    _run(conf_part)
    ck = sorted(os.listdir(roots_part["CHECKPOINT_ROOT"]))
    assert ck == ["rest_t00024_mpi000000.ckpt"]
    # ... whose outputs are removed, then the run resumed from step 24
    for f in os.listdir(roots_part["OUTPUT_ROOT"]):
        if "_n00003" in f or f.startswith("seismo"):
            os.remove(os.path.join(roots_part["OUTPUT_ROOT"], f))
    # the group holding step 24 is re-read from the file written at the checkpoint: put
    # those files back to their state at the checkpoint (frame of step 24 only), as a
    # crash right after the checkpoint would leave them
    for f in ("sgt_002_mpi000000_n00002.nc", "vel_002_mpi000000_n00002.nc"):
        _keep_records(os.path.join(roots_part["OUTPUT_ROOT"], f), 1)
    from fwant_gb300 import inputs
    m = small_model("surface")
    inputs.write_conf(conf_part, m, NT, roots_part, snaps=SNAPS, checkpoint_tinv=12, run_from_checkpoint=24)
    _run(conf_part)
    for f in sorted(os.listdir(roots_full["OUTPUT_ROOT"])):
        a, _ = _read(os.path.join(roots_full["OUTPUT_ROOT"], f))
        b, _ = _read(os.path.join(roots_part["OUTPUT_ROOT"], f))
        for k in a:
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"{f}:{k}")
    shutil.rmtree(str(tmp_path), ignore_errors=True)


def test_urgent_checkpoint_file_and_step_log(native_lib, tmp_path):
    """The urgent-checkpoint control file (re-read every 10 steps: checkpoint step, sync
    step, new nt) and the per-step run-time log (fnm_log).  A run configured for nt = 30
    whose control file asks for nt = 44 and a checkpoint at step 20 runs 48 steps (whole
    8-step blocks past nt = 44), writes that checkpoint, and its seismograms equal a run
    configured for nt = 44 from the start; a missing control file stops the run."""
    base = os.path.join(str(tmp_path), "base")
    dyn = os.path.join(str(tmp_path), "dyn")
    os.makedirs(base)
    os.makedirs(dyn)
    from fwant_gb300 import inputs
    m = small_model("surface")
    _, conf_b, roots_b = _prepare(base)
    inputs.write_conf(conf_b, m, 44, roots_b, snaps=SNAPS)
    _run(conf_b)
    _, conf_d, roots_d = _prepare(dyn)
    urgent = os.path.join(dyn, "urgent.txt")
    log = os.path.join(dyn, "run.log")
    with open(urgent, "w") as f:
        f.write("20 0 44\n")
    with open(conf_d, "a") as f:
        f.write(f"urgent_checkpoint = {urgent}\nfnm_log = {log}\n")
    r = _run(conf_d)
    assert "reset nt to 44" in r.stdout
    assert sorted(os.listdir(roots_d["CHECKPOINT_ROOT"])) == ["rest_t00020_mpi000000.ckpt"]
    a, _ = _read(os.path.join(roots_b["OUTPUT_ROOT"], "seismo_mpi000000.nc"))
    b, _ = _read(os.path.join(roots_d["OUTPUT_ROOT"], "seismo_mpi000000.nc"))
    assert a["Vz"].shape[0] == b["Vz"].shape[0] == 48
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    lines = open(log).read().splitlines()
    steps = [ln for ln in lines if "step uses" in ln and ln.split()[0].isdigit()]
    assert len(steps) == 48 and steps[-1].split()[0] == "48"
    assert lines[0].strip() == "# seis3d_wave run time log" and "the total run time is" in open(log).read()
    os.remove(urgent)
    r = subprocess.run([EXE, conf_d], capture_output=True, text=True)
    assert r.returncode != 0 and "urgent" in r.stderr
    shutil.rmtree(str(tmp_path), ignore_errors=True)
