"""`fwant_ker --info`, the kernel statistics of SI_ker2info (code/srcF.kernel/SI_ker2info.F90),
on the GPU end to end through files: kernel files of many picks (random volumes over a
snapshot's I J K, some directories used by several picks) listed by station and event
lists with comments, a station name longer than 8 characters, an event name longer than
20, an event without picks and a pick with a filter name the kernel run would refuse; the
kerinfo_ file equals the restatement (oracle/kinfo_oracle.py) bit for bit: sums, counts,
every record's counts and name characters, the thresholds.  A missing kernel file stops the
program; a snapshot series without stresses writes nothing."""
import os
import subprocess

import numpy as np
import pytest

from helpers import small_model

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KER = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_ker")
SNAPS = [((1, 2, 1), (9, 7, 5), (1, 1, 2), 2, 5, "T"), ((1, 1, 1), (4, 4, 4), (1, 1, 1), 2, 5, "V")]
NAMES = ("phase_Vp", "amplitude_Vp", "phase_Vs", "amplitude_Vs")
SHAPE = (5, 7, 9)                  # (K, J, I) of snapshot 1
TH = (0.8, 1.1, 1.6, 0.5)


def _write_kernel(path, vols):
    from scipy.io import netcdf_file
    with netcdf_file(path, "w") as f:
        f.createDimension("I", SHAPE[2])
        f.createDimension("J", SHAPE[1])
        f.createDimension("K", SHAPE[0])
        f.title = b"Finite frequency kernel"
        for n, v in zip(NAMES, vols):
            f.createVariable(n, "f4", ("K", "J", "I"))[:] = v


def _read(path):
    from scipy.io import netcdf_file
    with netcdf_file(path, "r", mmap=False) as f:
        return {k: np.array(v[:]) for k, v in f.variables.items()}, dict(f._attributes)


@pytest.fixture(scope="module")
def case(tmp_path_factory, native_lib):
    pytest.importorskip("scipy")
    from fwant_gb300 import inputs
    tmp = str(tmp_path_factory.mktemp("kinfo"))
    m = small_model("surface")
    main = os.path.join(tmp, "SeisFD3D.conf")
    roots = {k: tmp for k in ("GRID_ROOT", "MEDIA_ROOT", "SOURCE_ROOT", "STATION_ROOT", "OUTPUT_ROOT")}
    inputs.write_conf(main, m, 40, roots, snaps=SNAPS)
    rng = np.random.default_rng(31)
    vols = {}
    for d in "ABCDEFG":
        os.makedirs(os.path.join(tmp, "k", d))
        # heavy-tailed values with exact zeros and exact threshold values mixed in
        v = [(rng.standard_t(3, size=SHAPE) * 0.7).astype(np.float32) for _ in range(4)]
        for q in range(4):
            v[q][rng.random(SHAPE) < 0.1] = 0.0
            v[q][rng.random(SHAPE) < 0.05] = np.float32(TH[q]) * rng.choice([-1, 1])
        _write_kernel(os.path.join(tmp, "k", d, "kernel_001_mpi000000_n00000.nc"), v)
        vols[d] = v
    kd = lambda d: os.path.join(tmp, "k", d)  # noqa: E731
    rot = " ".join(["1.0", "0.0", "0.0", "0.0", "1.0", "0.0", "0.0", "0.0", "1.0"])
    syn = ["syn_x.txt", "syn_y.txt", "syn_z.txt"]   # listed, never read

    def event(name, comps):
        lines = [f"{name} " + " ".join(str(len(c)) for c in comps) + " " + rot] + syn
        for c in comps:
            for filt, d in c:
                lines += ["# a comment between picks", f"1 {filt} 1.5 9.0 {kd(d)}"]
        return lines

    ev1 = event("EV01", [[("P2", "A")], [], [("N", "B"), ("P1", "C")], [], [], [("P2", "A")]]) + \
        ["# comment"] + event("EV02", [[], [("N", "D")], [], [], [], []]) + \
        event("EV03", [[], [], [], [], [], []]) + \
        event("AN_EVENT_NAME_LONGER_THAN_20", [[("XX", "E")], [("N", "F")], [], [], [], []])
    ev2 = event("EV01", [[("N", "G")], [("N", "A")], [], [("N", "B")], [], []]) + \
        event("EV04", [[("N", "C"), ("N", "D"), ("N", "E")], [], [], [], [], []])
    ev3 = event("EV05", [[], [], [("N", "F")], [], [], [("N", "G")]]) + event("EV06", [[("N", "A")], [], [], [], [], []])
    for name, lines in (("ev1.lst", ev1), ("ev2.lst", ev2), ("ev3.lst", ev3)):
        with open(os.path.join(tmp, name), "w") as f:
            f.write("\n".join(lines) + "\n")
    sta = os.path.join(tmp, "sta.lst")
    with open(sta, "w") as f:
        f.write(f"# station  event list\nST01 {tmp}/ev1.lst\n  LONGSTATN {tmp}/ev2.lst\n\nST03 {tmp}/ev3.lst\n")
    conf = os.path.join(tmp, "TomoKernel.conf")
    with open(conf, "w") as f:
        f.write(f"MAIN_CONF = {main}\nsnap_id = 1\n")
    out = os.path.join(tmp, "info")
    os.makedirs(out)
    th = " ".join(repr(float(np.float32(t))) for t in TH)
    r = subprocess.run([KER, "--info", conf], input=f"{sta}\n{out}\n{th}\n0 0 0\n", capture_output=True, text=True,
                       cwd=tmp)
    assert r.returncode == 0, r.stdout + r.stderr
    # the same inputs, parsed by hand for the restatement
    stations = [
        ("ST01", [("EV01", ["A", "B", "C", "A"]), ("EV02", ["D"]), ("EV03", []),
                  ("AN_EVENT_NAME_LONGER_THAN_20", ["E", "F"])]),
        ("LONGSTATN", [("EV01", ["G", "A", "B"]), ("EV04", ["C", "D", "E"])]),
        ("ST03", [("EV05", ["F", "G"]), ("EV06", ["A"])]),
    ]
    return dict(tmp=tmp, conf=conf, sta=sta, out=out, vols=vols, stations=stations, stdout=r.stdout)


def test_kerinfo_file_equals_the_restatement(case):
    from oracle import kinfo_oracle as KI
    info = KI.run(case["stations"], TH, SHAPE, lambda d: case["vols"][d])
    got, att = _read(os.path.join(case["out"], "kerinfo_001_mpi000000_n00000.nc"))
    for q, name in enumerate(("Kap", "Kaq", "Kbp", "Kbq")):
        assert np.float32(att["threshold_" + name]) == np.float32(TH[q])
    nrec = info.records()
    assert nrec >= 3 and f"{nrec} records" in case["stdout"]
    for q, s in enumerate(("ap", "aq", "bp", "bq")):
        np.testing.assert_array_equal(got["S" + s], info.S[q].reshape(SHAPE), err_msg="S" + s)
        np.testing.assert_array_equal(got["N" + s], info.N[q].reshape(SHAPE), err_msg="N" + s)
        assert got["M" + s].shape == (nrec,) + SHAPE
        assert got["KSTNM" + s].shape == (nrec,) + SHAPE + (8,)
        assert got["KEVNM" + s].shape == (nrec,) + SHAPE + (20,)
        for r in range(nrec):
            np.testing.assert_array_equal(got["M" + s][r], info.rec_M[r][q].reshape(SHAPE), err_msg=f"M{s} {r}")
            for which, var, width in ((0, "KSTNM", 8), (1, "KEVNM", 20)):
                want = info.char_record(r, q, which).reshape(SHAPE + (width,))
                have = np.ascontiguousarray(got[var + s][r]).view(np.uint8).reshape(SHAPE + (width,))
                np.testing.assert_array_equal(have, want, err_msg=f"{var}{s} {r}")
    # the cases the file must show: names kept, refused (too long), refused record index 0
    assert np.any(info.N[1] > info.N[0])          # aq counted where ap never reached
    names = {bytes(c).rstrip(b"\0") for c in info.char_record(0, 0, 1)}
    assert b"EV01" in names and b"AN_EVENT_NAME_LONGER_THAN_20" not in names


def test_missing_kernel_file_stops(case):
    tmp = case["tmp"]
    with open(os.path.join(tmp, "ev_bad.lst"), "w") as f:
        f.write("EVX 1 0 0 0 0 0 1 0 0 0 1 0 0 0 1\na\nb\nc\n1 N 1.0 2.0 " + os.path.join(tmp, "nowhere") + "\n")
    with open(os.path.join(tmp, "sta_bad.lst"), "w") as f:
        f.write(f"ST01 {tmp}/ev_bad.lst\n")
    r = subprocess.run([KER, "--info", case["conf"]], input=f"{tmp}/sta_bad.lst\n{tmp}\n1 1 1 1\n0 0 0\n",
                       capture_output=True, text=True, cwd=tmp)
    assert r.returncode != 0 and "nowhere" in r.stderr


def test_series_without_stresses_writes_nothing(case):
    tmp = case["tmp"]
    conf = os.path.join(tmp, "TomoKernel_v.conf")
    with open(conf, "w") as f:
        f.write(f"MAIN_CONF = {tmp}/SeisFD3D.conf\nsnap_id = 2\n")
    out = os.path.join(tmp, "info_v")
    os.makedirs(out)
    r = subprocess.run([KER, "--info", conf], input=f"{case['sta']}\n{out}\n1 1 1 1\n0 0 0\n", capture_output=True,
                       text=True, cwd=tmp)
    assert r.returncode == 0, r.stderr
    assert "nothing to do" in r.stdout and os.listdir(out) == []


def test_api_against_the_restatement(native_lib):
    """fwant_kerinfo through the C ABI over 40 events (records grow past the first
    allocation of the record table): sums, counts and every record equal the restatement;
    tags 0 (names not stored) keep earlier names."""
    import fwant_gb300 as fw
    from oracle import kinfo_oracle as KI
    rng = np.random.default_rng(8)
    npts = 3001
    th = (0.3, 0.9, 1.4, 0.05)
    g = fw.KerInfo(npts, th)
    o = KI.KerInfo((npts,), th)
    sta_names = ["S1", "S2", "TOO_LONG_NAME"]
    evt_names = [f"E{e:02d}" for e in range(40)]
    for e in range(40):
        for _ in range(int(rng.integers(1, 4))):
            ks = [rng.normal(size=npts).astype(np.float32) for _ in range(4)]
            g.add_pick(ks)
            o.add_pick(ks)
        s = e % 3
        g.end_event(s + 1 if len(sta_names[s]) <= 8 else 0, e + 1 if e % 7 else 0)
        o.end_event(sta_names[s], evt_names[e] if e % 7 else "")
    S, N = g.totals()
    np.testing.assert_array_equal(S, o.S)
    np.testing.assert_array_equal(N, o.N)
    assert g.records() == o.records() > 16
    for r in range(o.records()):
        m, st, ev = g.record(r)
        np.testing.assert_array_equal(m, o.rec_M[r])
        want_s = np.vectorize(lambda x: 0 if x is None else sta_names.index(x) + 1, otypes=[np.int32])(o.rec_sta[r])
        want_e = np.vectorize(lambda x: 0 if x is None else evt_names.index(x) + 1, otypes=[np.int32])(o.rec_evt[r])
        np.testing.assert_array_equal(st, want_s)
        np.testing.assert_array_equal(ev, want_e)
    assert g.last_ms() >= 0.0
    g.close()
