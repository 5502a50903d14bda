"""`fwant_ker`, the station sensitivity-kernel program (SI_ker_sta) on the GPU, end to end
through files: four `fwant_wave` runs write the sgt_ snapshot series of a station's three
force components and of an event; `fwant_ker` reads them block by block with the
reference's TomoKernel.conf, filter files, station and event lists, and writes one kernel
file per pick.  Every kernel file equals the restatement's pipeline on the same SGTs
(stress2strain + sgt2scatter3 in FP64 accumulation, the component rotation, the pick's
filter and window) bit for bit after the cast to float32; the points outside the kernel
selection stay zero, a pick outside the time range writes no file, and a second run that
starts at a later block over the first run's files (first_run false) rewrites them
unchanged."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import LENFD, small_model

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WAVE = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_wave")
KER = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_ker")
ASSM = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_assm")
NT = 40                                  # 48 steps executed: 24 frames at tinv 2
SNAP = ((3, 4, 5), (6, 5, 4), (2, 2, 2), 2, 5, "T")
KNT = 20                                 # frames used: files n00001-n00004
SUB = dict(sub_start=(2, 1, 1), sub_count=(-1, 4, -1), sub_stride=(2, 1, 1), block_size=(2, 3, -1))
M0 = 1.0e15


def _read(path):
    from scipy.io import netcdf_file
    with netcdf_file(path, "r", mmap=False) as f:
        return {k: np.array(v[:]) for k, v in f.variables.items()}, dict(f._attributes)


def _wave_run(tmp, m, out_dir):
    from fwant_gb300 import inputs
    os.makedirs(tmp, exist_ok=True)
    os.makedirs(out_dir, exist_ok=True)
    inputs.write_inputs(m, tmp)
    roots = {k: tmp for k in ("GRID_ROOT", "MEDIA_ROOT", "SOURCE_ROOT", "STATION_ROOT")}
    roots["OUTPUT_ROOT"] = out_dir
    conf = os.path.join(tmp, "SeisFD3D.conf")
    inputs.write_conf(conf, m, NT, roots, snaps=[SNAP])
    r = subprocess.run([WAVE, conf], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return conf


def _sgt_series(out_dir):
    """(6, KNT, K, J, I) stresses of the snapshot series from its files."""
    frames = []
    n = 1
    while sum(f.shape[1] for f in frames) < KNT:
        v, _ = _read(os.path.join(out_dir, f"sgt_001_mpi000000_n{n:05d}.nc"))
        frames.append(np.stack([v[c] for c in ("Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz")]))
        n += 1
    return np.concatenate(frames, axis=1)[:, :KNT]


def _window(t, t1, t2, kdt):
    """Pick window (SI_ker_sta.F90:676-704) over the synthetic's times t; the range is
    kdt .. knt kdt.  None when the pick is skipped."""
    knt = t.size
    tmin, tmax = kdt, np.float32(knt) * kdt
    if t1 > tmax or t2 < tmin:
        return None
    nt1 = 1 if t1 <= tmin else int(np.flatnonzero(t <= t1)[np.argmax(t[t <= t1])]) + 1
    nt2 = knt if t2 >= tmax else int(np.flatnonzero(t >= t2)[np.argmin(t[t >= t2])]) + 1
    return nt1, nt2


@pytest.fixture(scope="module")
def runs(tmp_path_factory, native_lib):
    signal = pytest.importorskip("scipy.signal")
    from fwant_gb300 import inputs
    tmp = str(tmp_path_factory.mktemp("ker"))
    sgt_root, evt_root = os.path.join(tmp, "SGT"), os.path.join(tmp, "EVT")
    # the station's three force runs and the event run share grid and medium
    for c, name in enumerate(("FX", "FY", "FZ")):
        m = small_model("surface")
        for q, f in enumerate((m.fx, m.fy, m.fz)):
            f[:] = np.float32(1.0e15) if q == c else np.float32(0.0)
        _wave_run(os.path.join(tmp, "run_" + name), m, os.path.join(sgt_root, "STA", name))
    main = _wave_run(os.path.join(tmp, "run_ev"), small_model("buried"), os.path.join(evt_root, "EV1", "OUT"))
    os.symlink(os.path.join(evt_root, "EV1"), os.path.join(evt_root, "EV2"))  # a second event, same SGTs
    m = small_model("surface")
    kdt = np.float32(SNAP[3]) * np.float32(m.stept)
    t = np.float32(np.arange(1, KNT + 1)) * kdt
    rng = np.random.default_rng(12)
    syn = []
    for c in range(4):
        v = rng.normal(size=KNT).astype(np.float32)
        u = (np.cumsum(v) * kdt).astype(np.float32)
        p = os.path.join(tmp, f"syn{c}.txt")
        inputs.write_synthetic(p, t, v, u)
        syn.append((p, v, u))
    b, a = signal.butter(2, [0.15, 0.45], btype="band")
    fb, fa = inputs.write_filter_file(os.path.join(tmp, "bp1.txt"), b, a)
    kd = lambda name: os.path.join(tmp, "kernels", name)  # noqa: E731
    picks1 = [[(1, "P2", 2.5 * kdt, 15.2 * kdt, kd("A"))],
              [(1, "N", 100 * kdt, 200 * kdt, kd("F"))],                       # after the series: skipped
              [(2, "N", 0.5 * kdt, 30 * kdt, kd("B")), (1, "P1", 3 * kdt, 16 * kdt, kd("C"))],
              [(2, "N", 1.5 * kdt, 12 * kdt, kd("D"))],
              [],
              [(1, "P2", 4 * kdt, 19 * kdt, kd("E"))]]
    picks2 = [[], [(2, "N", 2 * kdt, 18 * kdt, kd("G"))], [], [], [], []]
    th = 0.6
    rot = np.array([[np.cos(th), -np.sin(th), 0.0], [np.sin(th), np.cos(th), 0.0], [0.0, 0.0, 1.0]])
    events = [dict(name="EV1", picks=picks1, rot=rot, syn=[s[0] for s in syn[:3]]),
              dict(name="EV2", picks=picks2, rot=np.eye(3), syn=[syn[3][0], syn[3][0], syn[3][0]])]
    for e in events:
        for comp in e["picks"]:
            for p in comp:
                os.makedirs(p[4], exist_ok=True)
    evt = os.path.join(tmp, "evt.lst")
    inputs.write_event_list(evt, events)
    sta = os.path.join(tmp, "sta.lst")
    with open(sta, "w") as f:
        f.write(f"# station  event list\nSTA {evt}\n")
    kroots = dict(SGT_ROOT=sgt_root, SGT_STAX="FX", SGT_STAY="FY", SGT_STAZ="FZ", EVENT_ROOT=evt_root,
                  EVENT_OUTD="OUT")
    conf = os.path.join(tmp, "TomoKernel.conf")
    inputs.write_tomo_conf(conf, main, 1, kroots, KNT, M0, filter_files=[os.path.join(tmp, "bp1.txt"), "none"], **SUB)
    r = subprocess.run([KER, conf], input=f"{sta}\n0 0 0\n", capture_output=True, text=True, cwd=tmp)
    assert r.returncode == 0, r.stderr
    assert "t1>Tmax" in r.stderr
    return dict(tmp=tmp, m=m, kdt=kdt, t=t, syn=syn, filt=(fb, fa), events=events, conf=conf, sta=sta,
                sgt_root=sgt_root, evt_root=evt_root, kd=kd, stdout=r.stdout)


def _selection(m):
    """0-based sample indices (per axis) of the kernel selection in the snapshot's grid and
    lambda, mu at those points in file (K, J, I) layout."""
    subs, subc, subt = SNAP[0], SNAP[1], SNAP[2]
    sel = []
    for d in range(3):
        st, cnt, sd = SUB["sub_start"][d], SUB["sub_count"][d], SUB["sub_stride"][d]
        n = (subc[d] - st) // sd + 1
        if cnt != -1:
            n = min(n, cnt)
        sel.append(np.arange(st - 1, st - 1 + n * sd, sd))
    gi = [LENFD + subs[d] - 1 + sel[d] * subt[d] for d in range(3)]
    lam = m.lam[np.ix_(*gi)].transpose(2, 1, 0)
    mu = m.mu[np.ix_(*gi)].transpose(2, 1, 0)
    return sel, lam, mu


def _expected(R, oracle_mod, param=0, eq=False):
    """Kernels of every pick over all selected points, float32, in file (K, J, I) layout
    (param 0 Vp/Vs kernels, 1 lambda/mu kernels; eq: the Z-force SGT moved 9 frames
    earlier, SI_ker_EQ)."""
    m, kdt, t = R["m"], R["kdt"], R["t"]
    subs, subc, subt = SNAP[0], SNAP[1], SNAP[2]
    # selected sample indices (0-based) per axis: start, stride, count of the kernel selection
    sel = []
    for d in range(3):
        st, cnt, sd = SUB["sub_start"][d], SUB["sub_count"][d], SUB["sub_stride"][d]
        n = (subc[d] - st) // sd + 1
        if cnt != -1:
            n = min(n, cnt)
        sel.append(np.arange(st - 1, st - 1 + n * sd, sd))
    si, sj, sk = sel
    # media at those points (grid index with ghosts: first snapshot point + sample x stride)
    gi = [LENFD + subs[d] - 1 + sel[d] * subt[d] for d in range(3)]
    lam = m.lam[np.ix_(*gi)].transpose(2, 1, 0).reshape(-1)
    mu = m.mu[np.ix_(*gi)].transpose(2, 1, 0).reshape(-1)

    def block(series):  # (6, KNT, K, J, I) -> (6, KNT, points) with i fastest
        return np.ascontiguousarray(series[:, :, sk][:, :, :, sj][:, :, :, :, si].reshape(6, KNT, -1))
    rs = [block(_sgt_series(os.path.join(R["sgt_root"], "STA", c))) for c in ("FX", "FY", "FZ")]
    if eq:  # eoshift(., shift=9) along time (SI_ker_EQ.F90:580-586)
        rs[2] = np.concatenate([rs[2][:, 9:], np.zeros_like(rs[2][:, :9])], axis=1)
    ss = block(_sgt_series(os.path.join(R["evt_root"], "EV1", "OUT")))
    dt = float(kdt)
    m0 = float(np.float32(M0))
    fb, fa = R["filt"]
    out = {}
    for e, syn in ((R["events"][0], R["syn"][:3]), (R["events"][1], [R["syn"][3]] * 3)):
        rot_any = any(len(p) for p in e["picks"][3:])
        ud = [len(e["picks"][c]) > 0 or rot_any for c in range(3)]
        scat = oracle_mod.sgt2scatter3(lam, mu, [rs[c] if ud[c] else None for c in range(3)], ss, dt, mode=1,
                                       param=param)
        V = [s[1].copy() for s in syn]
        U = [s[2].copy() for s in syn]
        rot = np.asarray(e["rot"], np.float32).reshape(3, 3)
        for ncmp in range(1, 7):
            if ncmp == 4 and rot_any:
                for W in (V, U):
                    w0, w1, w2 = W[0].copy(), W[1].copy(), W[2].copy()
                    for c in range(3):
                        W[c] = (w0 * rot[0, c] + w1 * rot[1, c]) + w2 * rot[2, c]
                r64 = rot.astype(np.float64)
                for grp in ((0, 1, 2), (3, 5, 4)):
                    v = [scat[q].copy() for q in grp]
                    for c in range(3):
                        scat[grp[c]] = (v[0] * r64[0, c] + v[1] * r64[1, c]) + v[2] * r64[2, c]
            comp = (ncmp - 1) % 3
            sa, sb = ((0, 3), (1, 5), (2, 4))[comp]
            for band, filt, t1, t2, d in e["picks"][ncmp - 1]:
                w = _window(t, np.float32(t1), np.float32(t2), kdt)
                if w is None:
                    out[d] = None
                    continue
                if filt == "N":
                    k = oracle_mod.scatter2kernel(V[comp], U[comp], scat[sa], scat[sb], dt, w[0], w[1], m0, mode=1)
                else:
                    k = oracle_mod.scatter2kernel_filtered(V[comp], U[comp], scat[sa], scat[sb], dt, w[0], w[1], m0,
                                                           fb, fa, 1 if filt == "P1" else 2)
                full = []
                for q in range(4):
                    a = np.zeros((subc[2], subc[1], subc[0]), np.float32)
                    a[np.ix_(sk, sj, si)] = np.asarray(k[q], np.float64).astype(np.float32).reshape(
                        sk.size, sj.size, si.size)
                    full.append(a)
                out[d] = full
    return out


NAMES = ("phase_Vp", "amplitude_Vp", "phase_Vs", "amplitude_Vs")


def test_kernel_files_equal_the_restatement(runs, oracle_mod):
    want = _expected(runs, oracle_mod)
    assert len(want) == 7
    for d, w in want.items():
        path = os.path.join(d, "kernel_001_mpi000000_n00000.nc")
        if w is None:
            assert not os.path.exists(path)
            continue
        got, att = _read(path)
        assert att["title"] == b"Finite frequency kernel"
        for q, name in enumerate(NAMES):
            assert got[name].shape == (SNAP[1][2], SNAP[1][1], SNAP[1][0])
            np.testing.assert_array_equal(got[name], w[q], err_msg=f"{d}:{name}")
            assert np.any(w[q])


def test_assembly_of_the_kernel_files(runs):
    """The kernel files this program writes are the assembly's input: fwant_assm (SI_ker2assm)
    run on them writes the compact rows of the restatement's projection byte for byte."""
    from scipy.io import netcdf_file

    import assm_case as ac
    from fwant_gb300 import inputs
    from oracle import assm_oracle as A
    tmp = runs["tmp"]
    shape = tuple(SNAP[1])
    volume, npix, pixs = ac.blocks(shape, brick=(2, 2, 2), seed=5)
    nblk, max_pix = volume.shape[1], volume.shape[0]
    blk = os.path.join(tmp, "blocks.nc")
    with netcdf_file(blk, "w", version=1) as f:
        f.createDimension("block", nblk)
        f.createDimension("max_pix", max_pix)
        f.createDimension("geo", 3)
        f.createVariable("volume", "f4", ("block", "max_pix"))[:] = volume.T
        f.createVariable("num_of_pix", "i4", ("block",))[:] = npix
        f.createVariable("indx_of_pix", "i4", ("block", "max_pix", "geo"))[:] = pixs.transpose(2, 1, 0)
    # the picks that have kernel files (the one after the series was skipped)
    events = [dict(e, picks=[[p for p in comp if os.path.exists(os.path.join(p[4], "kernel_001_mpi000000_n00000.nc"))]
                             for comp in e["picks"]]) for e in runs["events"]]
    evt = os.path.join(tmp, "evt_assm.lst")
    inputs.write_event_list(evt, events)
    sta = os.path.join(tmp, "sta_assm.lst")
    with open(sta, "w") as f:
        f.write(f"STA {evt}\n")
    spool = os.path.join(tmp, "spool")
    os.makedirs(spool)
    r = subprocess.run([ASSM, runs["conf"]], input=f"{sta}\n{blk}\n{spool}\n1.0 1.0 1.0 1.0\n0.0 0.0 0.0 0.0\n",
                       capture_output=True, text=True, cwd=tmp)
    assert r.returncode == 0, r.stdout + r.stderr
    dirs = [p[4] for e in events for comp in e["picks"] for p in comp]
    assert len(dirs) == 6
    for d in dirs:
        ker, _ = _read(os.path.join(d, "kernel_001_mpi000000_n00000.nc"))
        part = d.lstrip("./").replace("/", "_")
        for name, tag in (("phase_Vp", "Kap"), ("phase_Vs", "Kbp")):
            B = A.project(ker[name].transpose(2, 1, 0), volume, npix, pixs)
            idx, val = A.compact(B, 1.0, 0.0)
            assert len(idx) > 0
            with open(os.path.join(spool, f"{part}.{tag}.unformat"), "rb") as f:
                assert f.read() == A.row_file_bytes(nblk, 0.0, idx, val), (d, tag)


def test_lamu_kernel_files_equal_the_restatement(runs, oracle_mod):
    """--lamu (SI_ker_sta_lamu): the same inputs give the lambda/mu kernels, written to
    kernel_lamu_NNN files under phase_la amplitude_la phase_mu amplitude_mu, equal to the
    restatement's; the Vp/Vs files of the same picks are left as they were."""
    before = {d: _read(os.path.join(d, "kernel_001_mpi000000_n00000.nc"))[0]
              for d in _expected(runs, oracle_mod) if os.path.exists(os.path.join(d, "kernel_001_mpi000000_n00000.nc"))}
    for e in runs["events"]:
        for comp in e["picks"]:
            for p in comp:
                os.makedirs(p[4], exist_ok=True)
    r = subprocess.run([KER, "--lamu", runs["conf"]], input=f"{runs['sta']}\n0 0 0\n", capture_output=True,
                       text=True, cwd=runs["tmp"])
    assert r.returncode == 0, r.stderr
    want = _expected(runs, oracle_mod, param=1)
    names = ("phase_la", "amplitude_la", "phase_mu", "amplitude_mu")
    for d, w in want.items():
        path = os.path.join(d, "kernel_lamu_001_mpi000000_n00000.nc")
        if w is None:
            assert not os.path.exists(path)
            continue
        got, _ = _read(path)
        for q, name in enumerate(names):
            np.testing.assert_array_equal(got[name], w[q], err_msg=f"{d}:{name}")
            assert np.any(w[q])
    for d, b in before.items():
        after, _ = _read(os.path.join(d, "kernel_001_mpi000000_n00000.nc"))
        for name in NAMES:
            np.testing.assert_array_equal(after[name], b[name])


def test_kernel_conversions(runs):
    """--convert lamu2vpvs, vpvs2kamu, lamu2kamu (SI_ker_lamu2vpvs, SI_ker_vpvs2kamu,
    SI_ker_lamu2kamu) over lambda/mu kernel files that --lamu wrote into fresh pick
    directories: every output block equals the restatement (oracle/kconv_oracle.py) applied
    to the input file with the block's lambda and mu, bit for bit; points outside the
    selection stay zero; lamu2vpvs then vpvs2kamu agrees with lamu2kamu to rounding; the
    skipped pick gets no file."""
    from fwant_gb300 import inputs
    from oracle import kconv_oracle as KC
    tmp = runs["tmp"]
    cd = lambda name: os.path.join(tmp, "conv", name)  # noqa: E731
    events = [dict(e, picks=[[(p[0], p[1], p[2], p[3], cd(os.path.basename(p[4]))) for p in comp]
                             for comp in e["picks"]]) for e in runs["events"]]
    dirs = sorted({p[4] for e in events for comp in e["picks"] for p in comp})
    for d in dirs:
        os.makedirs(d, exist_ok=True)
    evt = os.path.join(tmp, "evt_conv.lst")
    inputs.write_event_list(evt, events)
    sta = os.path.join(tmp, "sta_conv.lst")
    with open(sta, "w") as f:
        f.write(f"STA {evt}\n")

    def run(*args, stdin):
        r = subprocess.run([KER, *args, runs["conf"]], input=stdin, capture_output=True, text=True, cwd=tmp)
        assert r.returncode == 0, r.stdout + r.stderr
        return r

    run("--lamu", stdin=f"{sta}\n0 0 0\n")
    sel, lam, mu = _selection(runs["m"])
    ix = np.ix_(sel[2], sel[1], sel[0])
    lam_names = ("phase_la", "amplitude_la", "phase_mu", "amplitude_mu")
    kamu_names = ("phase_ka", "amplitude_ka", "phase_mu", "amplitude_mu")
    skipped = cd("F")

    def check(mode, in_file, in_names, out_file, out_names):
        run("--convert", mode, stdin=f"\n{sta}\n0 0 0\n")
        outs = {}
        for d in dirs:
            if d == skipped:
                assert not os.path.exists(os.path.join(d, out_file))
                continue
            src, _ = _read(os.path.join(d, in_file))
            got, att = _read(os.path.join(d, out_file))
            assert att["title"] == b"Finite frequency kernel"
            for ph in (0, 1):  # phase pair, amplitude pair
                a, b = KC.convert(mode, lam, mu, src[in_names[ph]][ix], src[in_names[2 + ph]][ix])
                for q, want in ((ph, a), (2 + ph, b)):
                    full = np.zeros(SNAP[1][::-1], np.float32)
                    full[ix] = want
                    np.testing.assert_array_equal(got[out_names[q]], full, err_msg=f"{mode} {d} {out_names[q]}")
                    assert np.any(want)
            outs[d] = got
        return outs

    check("lamu2vpvs", "kernel_lamu_001_mpi000000_n00000.nc", lam_names, "kernel_001_mpi000000_n00000.nc", NAMES)
    via = check("vpvs2kamu", "kernel_001_mpi000000_n00000.nc", NAMES, "kernel_kamu_001_mpi000000_n00000.nc",
                kamu_names)
    direct = check("lamu2kamu", "kernel_lamu_001_mpi000000_n00000.nc", lam_names, "kernel_001_mpi000000_n00000.nc",
                   NAMES)
    for d in via:
        for qa, qb in zip(kamu_names, NAMES):
            a, b = via[d][qa].astype(np.float64), direct[d][qb].astype(np.float64)
            np.testing.assert_allclose(a, b, rtol=0, atol=2e-6 * np.abs(b).max())


def test_eq_kernel_files_equal_the_restatement(runs, oracle_mod):
    """--eq (SI_ker_EQ): the station's Z-force SGT moved 9 frames earlier before the
    accumulation; every kernel file equals the restatement's on the shifted series, and the
    picks that use the Z component differ from the plain run's."""
    from fwant_gb300 import inputs
    tmp = runs["tmp"]
    ed = lambda name: os.path.join(tmp, "eq", name)  # noqa: E731
    events = [dict(e, picks=[[(p[0], p[1], p[2], p[3], ed(os.path.basename(p[4]))) for p in comp]
                             for comp in e["picks"]]) for e in runs["events"]]
    for e in events:
        for comp in e["picks"]:
            for p in comp:
                os.makedirs(p[4], exist_ok=True)
    evt = os.path.join(tmp, "evt_eq.lst")
    inputs.write_event_list(evt, events)
    sta = os.path.join(tmp, "sta_eq.lst")
    with open(sta, "w") as f:
        f.write(f"STA {evt}\n")
    r = subprocess.run([KER, "--eq", runs["conf"]], input=f"{sta}\n0 0 0\n", capture_output=True, text=True, cwd=tmp)
    assert r.returncode == 0, r.stderr
    want = _expected(dict(runs, events=events), oracle_mod, eq=True)
    plain = _expected(dict(runs, events=events), oracle_mod)
    differs = 0
    for d, w in want.items():
        path = os.path.join(d, "kernel_001_mpi000000_n00000.nc")
        if w is None:
            assert not os.path.exists(path)
            continue
        got, _ = _read(path)
        for q, name in enumerate(NAMES):
            np.testing.assert_array_equal(got[name], w[q], err_msg=f"{d}:{name}")
        differs += any(not np.array_equal(w[q], plain[d][q]) for q in range(4))
    assert differs >= 2


def test_resumed_blocks_rewrite_the_same_files(runs):
    """first_run false and block_from (2, 1, 1): the later blocks are recomputed into the
    existing files, which keep their content."""
    from fwant_gb300 import inputs
    before = {}
    for d in ("A", "E", "G"):
        before[d] = _read(os.path.join(runs["kd"](d), "kernel_001_mpi000000_n00000.nc"))[0]
    conf = os.path.join(runs["tmp"], "TomoKernel_resume.conf")
    kroots = dict(SGT_ROOT=runs["sgt_root"], SGT_STAX="FX", SGT_STAY="FY", SGT_STAZ="FZ",
                  EVENT_ROOT=runs["evt_root"], EVENT_OUTD="OUT")
    main = os.path.join(runs["tmp"], "run_ev", "SeisFD3D.conf")
    inputs.write_tomo_conf(conf, main, 1, kroots, KNT, M0, first_run=False, block_from=(2, 1, 1),
                           filter_files=[os.path.join(runs["tmp"], "bp1.txt"), "none"], **SUB)
    r = subprocess.run([KER, conf], input=f"{runs['sta']}\n0 0 0\n", capture_output=True, text=True, cwd=runs["tmp"])
    assert r.returncode == 0, r.stderr
    for d, b in before.items():
        got = _read(os.path.join(runs["kd"](d), "kernel_001_mpi000000_n00000.nc"))[0]
        for name in NAMES:
            np.testing.assert_array_equal(got[name], b[name])
    shutil.rmtree(os.path.join(runs["tmp"], "kernels"), ignore_errors=True)


def test_pair_kernel_files_equal_the_restatement(runs):
    """--pair, SI_ker_pair: one receiver (the station's Z-force SGT series) against the
    event's series, read block by block (2 x 3 x all points), kernels of five windows (both
    filter passes, no filter, two windows sharing a band and filter) written under the
    kernel_phase_Vp ... names; every file equals the restatement (oracle/kpair_oracle.py) of
    the whole snapshot bit for bit."""
    from oracle import kpair_oracle as KP
    R = runs
    tmp, m, kdt = R["tmp"], R["m"], R["kdt"]
    subs, subc, subt = SNAP[0], SNAP[1], SNAP[2]
    pd = lambda name: os.path.join(tmp, "pair", name)  # noqa: E731
    wins = [(1, 1, 2.5 * kdt, 15.2 * kdt, pd("A")), (1, 2, 3 * kdt, 17 * kdt, pd("B")),
            (1, 2, 1.5 * kdt, 12 * kdt, pd("C")), (2, 3, 2 * kdt, 18 * kdt, pd("D")),
            (1, 3, 4 * kdt, 19 * kdt, pd("E"))]
    for w in wins:
        os.makedirs(w[4], exist_ok=True)
    t, (_, v, u) = R["t"], R["syn"][0]
    syn = os.path.join(tmp, "pair_syn.txt")
    with open(syn, "w") as f:
        f.write(f"{KNT}\n" + "".join(f"{float(a)!r} {float(b)!r} {float(c)!r}\n" for a, b, c in zip(t, v, u)))
    main = os.path.join(tmp, "run_ev", "SeisFD3D.conf")
    conf = os.path.join(tmp, "TomoKernel_pair.conf")
    lines = [f"MAIN_CONF = {main}", f"SGT_ROOT = {os.path.join(R['sgt_root'], 'STA', 'FZ')}", f"SGT_M0 = {M0!r}",
             f"WAVE_ROOT = {os.path.join(R['evt_root'], 'EV1', 'OUT')}", "snap_id = 1", "block_size = 2 3 -1",
             f"fnm_syn = {syn}", "number_of_freqband = 2", f"number_of_measured = {len(wins)}", "<time_window>"]
    for band, filt, t1, t2, d in wins:
        lines += [f"{band} {filt} {float(np.float32(t1))!r} {float(np.float32(t2))!r}", d]
    lines += ["<filter_file>", os.path.join(tmp, "bp1.txt"), "none"]
    with open(conf, "w") as f:
        f.write("\n".join(lines) + "\n")
    r = subprocess.run([KER, "--pair", conf], input="0 0 0\n", capture_output=True, text=True, cwd=tmp)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"{len(wins) * 3 * 2} pair kernel blocks" in r.stdout     # 3 x 2 x 1 blocks
    # the restatement over every snapshot point
    gi = [LENFD + subs[d] - 1 + np.arange(subc[d]) * subt[d] for d in range(3)]
    lam = m.lam[np.ix_(*gi)].transpose(2, 1, 0).reshape(-1)
    mu = m.mu[np.ix_(*gi)].transpose(2, 1, 0).reshape(-1)
    rs = _sgt_series(os.path.join(R["sgt_root"], "STA", "FZ")).reshape(6, KNT, -1)
    ss = _sgt_series(os.path.join(R["evt_root"], "EV1", "OUT")).reshape(6, KNT, -1)
    sa, sb = KP.scatter_pair(lam, mu, rs, ss, float(kdt))
    fb, fa = R["filt"]
    t32 = np.asarray(t, np.float32)
    for band, filt, t1, t2, d in wins:
        t1, t2 = np.float32(t1), np.float32(t2)
        nt1 = int(np.flatnonzero(t32 <= t1)[-1]) + 1
        nt2 = int(np.flatnonzero(t32 >= t2)[0]) + 1
        mode = 0 if filt == 3 else filt
        want = KP.kernel_pair(v, u, sa, sb, float(kdt), nt1, nt2, M0, mode=mode, b=fb, a=fa)
        got, att = _read(os.path.join(d, "kernel_001_mpi000000_n00000.nc"))
        assert att["title"] == b"Finite frequency kernel"
        for q, name in enumerate(("kernel_phase_Vp", "kernel_amplitude_Vp", "kernel_phase_Vs",
                                  "kernel_amplitude_Vs")):
            w = np.asarray(want[q]).astype(np.float32).reshape(subc[2], subc[1], subc[0])
            np.testing.assert_array_equal(got[name], w, err_msg=f"{d} {name}")
            assert np.any(w)
