"""The kernel program's file handling without a GPU: strided sub-array reads and in-place
writes of NetCDF classic variables (nf90_get_var / nf90_put_var with start, count and
stride, as SI_ker_sta reads sgt_ blocks and writes kernel blocks) against numpy slicing of
scipy's view of the same file; and TomoKernel.conf, filter files, the station and event
lists and standard input parsed up to the first device call."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_ker")

netcdf = pytest.importorskip("scipy.io").netcdf_file


@pytest.fixture(scope="module")
def exe(native_lib):
    assert os.path.exists(EXE), "fwant_ker not built"
    return EXE


def _lst(v):
    return ",".join(str(int(x)) for x in v)


def _sample(path, nrec, n_record_vars):
    rng = np.random.default_rng(nrec + 7 * n_record_vars)
    fixed = rng.normal(size=(5, 6, 7)).astype("f4")
    recs = [rng.normal(size=(nrec, 5, 6, 7)).astype("f4") for _ in range(n_record_vars)]
    with netcdf(path, "w", version=2) as f:
        f.createDimension("time", None)
        for d, n in (("K", 5), ("J", 6), ("I", 7)):
            f.createDimension(d, n)
        f.createVariable("fixed", "f4", ("K", "J", "I"))[:] = fixed
        f.createVariable("dbl", "f8", ("K", "J", "I"))[:] = fixed.astype("f8") * 3.0
        for q, a in enumerate(recs):
            f.createVariable(f"T{q}", "f4", ("time", "K", "J", "I"))[:nrec] = a
    return fixed, recs


SLABS3 = [((0, 0, 0), (5, 6, 7), (1, 1, 1)), ((1, 2, 3), (2, 2, 2), (2, 3, 2)), ((4, 5, 6), (1, 1, 1), (1, 1, 1)),
          ((0, 1, 0), (3, 1, 4), (2, 4, 2))]


@pytest.mark.parametrize("nrec,nrv", [(4, 1), (6, 3)])
def test_strided_reads_match_numpy(nrec, nrv, exe, tmp_path):
    import json
    path = os.path.join(tmp_path, "s.nc")
    fixed, recs = _sample(path, nrec, nrv)
    for name, arr in (("fixed", fixed), ("dbl", fixed.astype("f8") * 3.0)):
        for st, ct, sd in SLABS3:
            out = subprocess.run([exe, "--nc-slab", path, name, _lst(st), _lst(ct), _lst(sd)], capture_output=True,
                                 text=True, check=True).stdout
            want = arr[tuple(slice(s, s + (c - 1) * d + 1, d) for s, c, d in zip(st, ct, sd))]
            np.testing.assert_array_equal(np.array(json.loads(out), np.float32), want.astype("f4").reshape(-1))
    for q, arr in enumerate(recs):
        for st, ct, sd in (((1, 0, 1, 2), (nrec - 1, 5, 3, 2), (1, 1, 2, 3)), ((nrec - 1, 4, 5, 6), (1, 1, 1, 1),
                                                                                 (1, 1, 1, 1))):
            out = subprocess.run([exe, "--nc-slab", path, f"T{q}", _lst(st), _lst(ct), _lst(sd)],
                                 capture_output=True, text=True, check=True).stdout
            want = arr[tuple(slice(s, s + (c - 1) * d + 1, d) for s, c, d in zip(st, ct, sd))]
            np.testing.assert_array_equal(np.array(json.loads(out), np.float32), want.reshape(-1))
    # outside the variable: refused
    r = subprocess.run([exe, "--nc-slab", path, "fixed", "4,0,0", "2,1,1", "1,1,1"], capture_output=True, text=True)
    assert r.returncode == 1 and "outside" in r.stderr


def test_strided_writes_in_place(exe, tmp_path):
    path = os.path.join(tmp_path, "w.nc")
    fixed, recs = _sample(path, 3, 2)
    want = fixed.copy()
    for st, ct, sd in SLABS3[1:]:
        subprocess.run([exe, "--nc-fill-slab", path, "fixed", _lst(st), _lst(ct), _lst(sd)], check=True)
        sl = tuple(slice(s, s + (c - 1) * d + 1, d) for s, c, d in zip(st, ct, sd))
        want[sl] = np.arange(1, int(np.prod(ct)) + 1, dtype=np.float32).reshape(ct)
    with netcdf(path, "r", mmap=False) as f:
        np.testing.assert_array_equal(f.variables["fixed"][:], want)
        np.testing.assert_array_equal(f.variables["dbl"][:], fixed.astype("f8") * 3.0)  # untouched
        for q, a in enumerate(recs):
            np.testing.assert_array_equal(f.variables[f"T{q}"][:], a)
    r = subprocess.run([exe, "--nc-fill-slab", path, "dbl", "0,0,0", "1,1,1", "1,1,1"], capture_output=True, text=True)
    assert r.returncode == 1 and "not a fixed-size float" in r.stderr


def _kernel_setup(tmp_path, knt=20):
    """SeisFD3D.conf + media of the small test model, TomoKernel.conf, a filter file, a
    station list and an event list; no SGT files."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import small_model

    from fwant_gb300 import inputs
    signal = pytest.importorskip("scipy.signal")
    tmp = str(tmp_path)
    m = small_model("surface")
    inputs.write_inputs(m, tmp)
    roots = {k: tmp for k in ("GRID_ROOT", "MEDIA_ROOT", "SOURCE_ROOT", "STATION_ROOT", "OUTPUT_ROOT")}
    main = os.path.join(tmp, "SeisFD3D.conf")
    inputs.write_conf(main, m, 40, roots, snaps=[((3, 4, 5), (6, 5, 4), (2, 2, 2), 2, 5, "T")])
    b, a = signal.butter(2, [0.15, 0.45], btype="band")
    inputs.write_filter_file(os.path.join(tmp, "bp1.txt"), b, a)
    kroots = dict(SGT_ROOT=os.path.join(tmp, "SGT"), SGT_STAX="FX", SGT_STAY="FY", SGT_STAZ="FZ",
                  EVENT_ROOT=os.path.join(tmp, "EVT"), EVENT_OUTD="OUT")
    conf = os.path.join(tmp, "TomoKernel.conf")
    inputs.write_tomo_conf(conf, main, 1, kroots, knt, 1.0e15, filter_files=[os.path.join(tmp, "bp1.txt"), "none"])
    kdt = np.float32(2) * np.float32(m.stept)
    t = np.float32(np.arange(1, knt + 1)) * kdt
    syn = os.path.join(tmp, "syn.txt")
    inputs.write_synthetic(syn, t, np.ones(knt), np.ones(knt))
    picks = [[(1, "P2", 2 * kdt, 9 * kdt, os.path.join(tmp, "kA"))], [], [], [], [], []]
    inputs.write_event_list(os.path.join(tmp, "evt.lst"),
                            [dict(name="EV1", picks=picks, rot=np.eye(3), syn=[syn, syn, syn])])
    with open(os.path.join(tmp, "sta.lst"), "w") as f:
        f.write("# station event-list\nSTA " + os.path.join(tmp, "evt.lst") + "\n")
    return conf, os.path.join(tmp, "sta.lst")


def test_kernel_program_inputs_before_the_gpu(exe, tmp_path):
    conf, sta = _kernel_setup(tmp_path)

    def run(stdin, c=conf):
        return subprocess.run([exe, c], input=stdin, capture_output=True, text=True, cwd=str(tmp_path))

    # a complete set of inputs gets as far as the SGT files of the first block (not written here)
    r = run(f"{sta}\n0 0 0\n")
    assert r.returncode == 1 and ("sgt_001_mpi000000_n00001.nc" in r.stderr or "sgtker_create" in r.stderr), r.stderr
    # standard input, configuration and list errors
    assert "rank id must be 0 0 0" in run(f"{sta}\n1 0 0\n").stderr
    assert "rank id" in run(f"{sta}\n").stderr
    text = open(conf).read()
    for bad, msg in ((text.replace("snap_id = 1", "snap_id = 2"), "snap_002 missing"),
                     (text.replace("SGT_M0", "SGT_MX"), "key SGT_M0"),
                     (text.replace("first_run = .true.", "first_run = maybe"), "not a logical"),
                     (text.replace("number_of_freqband = 2", "number_of_freqband = 3"), "fewer filter files"),
                     (text.replace("block_size = -1 -1 -1", "block_size = 0 -1 -1"), "block_size")):
        open(conf, "w").write(bad)
        r = run(f"{sta}\n0 0 0\n")
        assert r.returncode == 1 and msg in r.stderr, (msg, r.stderr)
    open(conf, "w").write(text)
    evt = os.path.join(tmp_path, "evt.lst")
    good = open(evt).read()
    open(evt, "w").write(good.replace(" P2 ", " P3 "))
    assert "pickfilt error" in run(f"{sta}\n0 0 0\n").stderr
    lines = good.splitlines()
    open(evt, "w").write("\n".join(lines[:4]) + "\n")  # the pick line missing
    assert "pick line missing" in run(f"{sta}\n0 0 0\n").stderr
    open(evt, "w").write(good.replace("\n1 P2", "\n3 P2"))  # band 3 of 2
    assert "frequency band id overflow" in run(f"{sta}\n0 0 0\n").stderr
