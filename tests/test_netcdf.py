"""NetCDF classic files and SeisFD3D.conf: the program's reader and writer against an
independent implementation (scipy.io.netcdf_file), on files with every element type,
fixed and record variables, one and several record variables, and global attributes;
and the configuration parsing of `fwant_wave` up to the point where it needs a GPU."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_wave")

netcdf = pytest.importorskip("scipy.io").netcdf_file


@pytest.fixture(scope="module")
def exe(native_lib):
    assert os.path.exists(EXE), "fwant_wave not built"
    return EXE


def _write_sample(path, nrec, n_record_vars, version):
    rng = np.random.default_rng(nrec * 10 + n_record_vars)
    ref = {}
    with netcdf(path, "w", version=version) as f:
        f.createDimension("time", None)  # (scipy wants the record dimension first)
        f.createDimension("I", 5)
        f.createDimension("J", 3)
        f.title = b"sample file"
        f.ints = np.array([1, -2, 3], np.int32)
        f.scale = np.float32(2.5)
        for name, typ in (("b", "i1"), ("s", "i2"), ("i", "i4"), ("f", "f4"), ("d", "f8")):
            a = rng.integers(-100, 100, size=(3, 5)).astype(typ) if typ[0] == "i" else \
                rng.normal(size=(3, 5)).astype(typ)
            v = f.createVariable(name, typ, ("J", "I"))
            v[:] = a
            ref[name] = a
        for r in range(n_record_vars):
            a = rng.normal(size=(nrec, 3)).astype("f4")
            v = f.createVariable(f"rec{r}", "f4", ("time", "J"))
            v[:nrec] = a
            ref[f"rec{r}"] = a
        if n_record_vars:
            t = np.arange(nrec, dtype="i2")  # a short record variable: 2-byte slices
            v = f.createVariable("tshort", "i2", ("time",))
            v[:nrec] = t
            ref["tshort"] = t
    return ref


@pytest.mark.parametrize("nrec,nrv,version", [(0, 0, 1), (4, 1, 1), (7, 3, 1), (5, 2, 2)])
def test_reader_and_writer_agree_with_scipy(nrec, nrv, version, exe, tmp_path):
    src = os.path.join(tmp_path, "a.nc")
    ref = _write_sample(src, nrec, nrv, version)
    dump = json.loads(subprocess.run([exe, "--nc-dump", src], capture_output=True, text=True, check=True).stdout)
    assert dump["dims"]["I"] == 5 and dump["dims"]["J"] == 3 and dump["dims"]["time"] == 0
    for name, a in ref.items():
        assert dump["vars"][name]["count"] == a.size
        assert dump["vars"][name]["sum"] == pytest.approx(float(np.asarray(a, np.float64).sum()), rel=1e-12, abs=1e-9)
    dst = os.path.join(tmp_path, "b.nc")
    subprocess.run([exe, "--nc-copy", src, dst], check=True)
    with netcdf(dst, "r", mmap=False) as g:
        assert g.title == b"sample file"
        np.testing.assert_array_equal(g.ints, [1, -2, 3])
        assert float(g.scale) == 2.5
        for name, a in ref.items():
            np.testing.assert_array_equal(g.variables[name][:], a)


def test_damaged_file_is_refused(exe, tmp_path):
    p = os.path.join(tmp_path, "bad.nc")
    open(p, "wb").write(b"CDF\x01" + b"\xff" * 40)
    r = subprocess.run([exe, "--nc-dump", p], capture_output=True, text=True)
    assert r.returncode == 1 and "damaged" in r.stderr
    open(p, "wb").write(b"HDF5 not classic")
    r = subprocess.run([exe, "--nc-dump", p], capture_output=True, text=True)
    assert r.returncode == 1 and "not a NetCDF classic file" in r.stderr


def _setup(tmp_path):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import small_model

    from fwant_gb300 import inputs
    m = small_model("surface")
    inputs.write_inputs(m, str(tmp_path))
    roots = {k: str(tmp_path) for k in ("GRID_ROOT", "MEDIA_ROOT", "SOURCE_ROOT", "STATION_ROOT", "OUTPUT_ROOT")}
    return m, inputs, roots


def test_input_files_follow_the_reference_schema(tmp_path):
    m, inputs, _ = _setup(tmp_path)
    with netcdf(os.path.join(tmp_path, "media_mpi000000.nc"), "r", mmap=False) as f:
        assert f.variables["mu"].dimensions == ("K", "J", "I")
        np.testing.assert_array_equal(f.variables["mu"][:].transpose(2, 1, 0), m.mu)
    with netcdf(os.path.join(tmp_path, "station_mpi000000.nc"), "r", mmap=False) as f:
        assert f.dimensions["num_pt"] is None  # the record dimension, as seis3d_station writes it
        np.testing.assert_array_equal(f.variables["indx"][:], m.recv_indx)
        assert int(f.tinv) == m.recv_tinv
    with netcdf(os.path.join(tmp_path, "source_mpi000000.nc"), "r", mmap=False) as f:
        assert int(f.number_of_force) == 1 and int(f.force_stf_id) == 200
        np.testing.assert_array_equal(f.variables["force_indx"][:], m.force_indx)


def test_conf_errors_before_the_gpu(exe, tmp_path):
    m, inputs, roots = _setup(tmp_path)
    conf = os.path.join(tmp_path, "SeisFD3D.conf")
    inputs.write_conf(conf, m, 16, roots, snaps=[((-1, -1, -2), (-1, -1, 1), (2, 2, 1), 4, 2, "V")])
    # a complete configuration passes parsing and the input files (then needs a device)
    r = subprocess.run([exe, conf], capture_output=True, text=True, cwd=tmp_path)
    assert "key" not in r.stderr and "variable" not in r.stderr, r.stderr
    # missing key, decomposed grid, missing input file
    text = open(conf).read()
    for bad, msg in ((text.replace("nk = ", "nkk = "), "key nk"), (text.replace("dims = 1 1 1", "dims = 2 1 1"), "dims"),
                     (text.replace("MEDIA_ROOT = " + roots["MEDIA_ROOT"], "MEDIA_ROOT = /nonexistent"),
                      "cannot open")):
        open(conf, "w").write(bad)
        r = subprocess.run([exe, conf], capture_output=True, text=True, cwd=tmp_path)
        assert r.returncode == 1 and msg in r.stderr, (msg, r.stderr)
