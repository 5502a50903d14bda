"""Sensitivity-kernel accumulation on the GPU against the CPU restatement.

* sgt2scatter3 and scatter2kernel in FP64 accumulation reproduce the restatement of the
  same arithmetic bit for bit (products of FP32 strains are exact in FP64, every sum runs
  in the same order, fma rounds once);
* against the reference's FP32 arithmetic they agree to FP32 rounding (1e-4 relative L2);
* SGT frames recorded on the device equal the snapshots of the same steps, and feeding a
  solver's record directly gives the same kernels as feeding the frames from the host.
"""
import numpy as np
import pytest

from helpers import feed, small_model

pytestmark = pytest.mark.gpu


def _media(rng, npts):
    vp = rng.uniform(5800.0, 8000.0, npts)
    vs = vp / 1.73
    rho = rng.uniform(2600.0, 3300.0, npts)
    mu = (rho * vs * vs).astype(np.float32)
    lam = (rho * vp * vp - 2.0 * rho * vs * vs).astype(np.float32)
    return lam, mu


def _series(rng, npts, knt):
    t = np.arange(1, knt + 1)[:, None]
    f = rng.uniform(0.01, 0.05, size=(6, 1, npts))
    ph = rng.uniform(0, 2 * np.pi, size=(6, 1, npts))
    env = np.exp(-((t - knt / 2) / (knt / 4)) ** 2)
    noise = rng.normal(scale=0.05, size=(6, knt, npts))
    return (1e5 * (env * np.sin(2 * np.pi * f * t + ph) + noise)).astype(np.float32)


def test_lamu_scatter_bitwise_against_fp64_restatement(oracle_mod, native_lib):
    """set_param(1): the lambda/mu series of SI_ker_sta_lamu, bit for bit the restatement's."""
    import fwant_gb300 as fw
    rng = np.random.default_rng(77)
    npts, knt, dt = 41, 600, 0.1
    lam, mu = _media(rng, npts)
    r = [_series(rng, npts, knt) for _ in range(3)]
    s = _series(rng, npts, knt)
    k = fw.SgtKernel(npts, knt, dt)
    k.set_media(lam, mu)
    for c in range(3):
        k.set_sgt(c, r[c])
    k.set_sgt(3, s)
    with pytest.raises(fw.FwantError):
        k.set_param(2)
    k.set_param(1)
    k.scatter(7, 3, 590)
    want = oracle_mod.sgt2scatter3(lam, mu, r, s, dt, nt1=3, nt2=590, mode=1, param=1)
    for slot in range(6):
        np.testing.assert_array_equal(k.get_scatter(slot), want[slot], err_msg=f"slot {slot}")
        assert np.any(want[slot])
    k.set_param(0)
    k.scatter(4, 3, 590)
    vpvs = oracle_mod.sgt2scatter3(lam, mu, [None, None, r[2]], s, dt, nt1=3, nt2=590, mode=1)
    np.testing.assert_array_equal(k.get_scatter(2), vpvs[2])


# knt 700 spans two lag chunks (512) and three output chunks (256) of the device kernel
@pytest.mark.parametrize("flags,nt1,nt2", [(7, 1, 700), (5, 37, 651), (2, 300, 300)])
def test_scatter_bitwise_against_fp64_restatement(flags, nt1, nt2, oracle_mod, native_lib):
    import fwant_gb300 as fw
    rng = np.random.default_rng(flags * 100 + nt1)
    npts, knt, dt = 67, 700, 0.1
    lam, mu = _media(rng, npts)
    r = [_series(rng, npts, knt) if flags >> c & 1 else None for c in range(3)]
    s = _series(rng, npts, knt)
    k = fw.SgtKernel(npts, knt, dt)
    k.set_media(lam, mu)
    for c in range(3):
        if r[c] is not None:
            k.set_sgt(c, r[c])
    k.set_sgt(3, s)
    k.scatter(flags, nt1, nt2)
    want = oracle_mod.sgt2scatter3(lam, mu, r, s, dt, nt1=nt1, nt2=nt2, mode=1)
    ref32 = oracle_mod.sgt2scatter3(lam, mu, r, s, dt, nt1=nt1, nt2=nt2, mode=0)
    for slot in range(6):
        got = k.get_scatter(slot)
        np.testing.assert_array_equal(got, want[slot], err_msg=f"slot {slot}")
        if np.any(want[slot]):
            rel = np.linalg.norm(got - ref32[slot]) / np.linalg.norm(want[slot])
            assert rel < 1e-4, (slot, rel)
    # window kernels of every computed component
    v = rng.normal(size=knt).astype(np.float32)
    u = np.cumsum(v).astype(np.float32) * np.float32(dt)
    for ncmp in (1, 2, 3):
        if not flags >> (ncmp - 1) & 1:
            with pytest.raises(fw.FwantError):
                k.kernel(ncmp, v, u, nt1, nt2, 1.0e16)
            continue
        got = k.kernel(ncmp, v, u, nt1, nt2, 1.0e16)
        sa, sb = (0, 3) if ncmp == 1 else ((1, 5) if ncmp == 2 else (2, 4))
        exp = oracle_mod.scatter2kernel(v, u, want[sa], want[sb], dt, nt1, nt2, 1.0e16, mode=1)
        for g, e in zip(got, exp):
            np.testing.assert_array_equal(g, e)
        ref = oracle_mod.scatter2kernel(v, u, ref32[sa], ref32[sb], dt, nt1, nt2, 1.0e16, mode=0)
        for g, e in zip(got, ref):
            assert np.linalg.norm(g - e) / np.linalg.norm(g) < 1e-4


def test_argument_checks(native_lib):
    import fwant_gb300 as fw
    rng = np.random.default_rng(1)
    k = fw.SgtKernel(10, 20, 0.1)
    with pytest.raises(fw.FwantError) as e:
        k.scatter(1)
    assert e.value.code == 6  # media / SGT missing
    lam, mu = _media(rng, 10)
    bad = mu.copy()
    bad[3] = 0.0
    with pytest.raises(fw.FwantError) as e:
        k.set_media(lam, bad)
    assert e.value.code == 1
    k.set_media(lam, mu)
    k.set_sgt(3, _series(rng, 10, 20))
    with pytest.raises(fw.FwantError) as e:
        k.scatter(1)  # X receiver SGT missing
    assert e.value.code == 6
    k.set_sgt(0, _series(rng, 10, 20))
    for args in ((0,), (8,), (1, 0, 20), (1, 5, 21), (1, 9, 8)):
        with pytest.raises(fw.FwantError) as e:
            k.scatter(*args)
        assert e.value.code == 1
    k.scatter(1)
    v = np.ones(20, np.float32)
    with pytest.raises(fw.FwantError):
        k.kernel(4, v, v, 1, 20, 1.0)
    with pytest.raises(fw.FwantError):
        k.kernel(1, np.zeros(20, np.float32), v, 1, 20, 1.0)  # zero normalisation


def _sgt_model(kind, force):
    m = small_model(kind)
    m.fx[:] = 0.0
    m.fy[:] = 0.0
    m.fz[:] = 0.0
    (m.fx, m.fy, m.fz)[force][:] = np.float32(1.0e15)
    return m


def test_recorded_sgt_equals_snapshots_and_feeds_the_kernel(oracle_mod, native_lib):
    """Device SGT record == step-by-step snapshots == oracle fields (exact arithmetic);
    take_sgt from two solvers == set_sgt from their host frames."""
    import fwant_gb300 as fw
    subs, subc, subt = (5, 4, 6), (9, 7, 5), (2, 2, 3)
    tinv, nfr = 2, 12
    sims = []
    for kind, force in (("buried", 2), ("surface", 2)):
        m = _sgt_model(kind, force)
        met = oracle_mod.metric(m.x, m.y, m.z)
        g = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface, exact_arith=True), m, met, kind)
        g.set_sgt_record(subs, subc, subt, tinv, nfr)
        o = feed(oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface), m, met, kind)
        snaps = []
        for step in range(1, 2 * nfr + 5):
            g.run(1)
            o.run(1)
            if step % tinv == 0 and len(snaps) < nfr:
                snap = g.get_snapshot(subs, subc, subt, comps=("Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz"))
                # oracle field sub-volume, same (c, i, j, k) order
                ref = np.stack([o.get_field(c)[subs[0] - 1:subs[0] - 1 + subt[0] * subc[0]:subt[0],
                                               subs[1] - 1:subs[1] - 1 + subt[1] * subc[1]:subt[1],
                                               subs[2] - 1:subs[2] - 1 + subt[2] * subc[2]:subt[2]]
                                for c in ("Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz")])
                np.testing.assert_array_equal(snap, ref.astype(np.float32))
                snaps.append(snap.transpose(0, 3, 2, 1).reshape(6, -1))  # points i fastest
        rec = g.get_sgt()
        assert rec.shape == (6, nfr, int(np.prod(subc)))
        np.testing.assert_array_equal(rec, np.stack(snaps, axis=1))
        sims.append((g, m, rec))
    npts = int(np.prod(subc))
    m = sims[0][1]
    idx = [np.arange(subs[d] - 1, subs[d] - 1 + subt[d] * subc[d], subt[d]) for d in range(3)]
    lam = m.lam[np.ix_(*idx)].transpose(2, 1, 0).reshape(-1)
    mu = m.mu[np.ix_(*idx)].transpose(2, 1, 0).reshape(-1)
    kdt = tinv * m.stept
    a = fw.SgtKernel(npts, nfr, kdt)
    b = fw.SgtKernel(npts, nfr, kdt)
    for k in (a, b):
        k.set_media(lam, mu)
    a.take_sgt(2, sims[0][0])
    a.take_sgt(3, sims[1][0])
    b.set_sgt(2, sims[0][2])
    b.set_sgt(3, sims[1][2])
    a.scatter(4)
    b.scatter(4)
    for slot in (2, 4):
        np.testing.assert_array_equal(a.get_scatter(slot), b.get_scatter(slot))
        assert np.any(a.get_scatter(slot))
    want = oracle_mod.sgt2scatter3(lam, mu, [None, None, sims[0][2]], sims[1][2], kdt, mode=1)
    np.testing.assert_array_equal(a.get_scatter(2), want[2])
    # a solver without a record, or with too few frames, is refused
    short = fw.SgtKernel(npts, nfr + 1, kdt)
    short.set_media(lam, mu)
    with pytest.raises(fw.FwantError) as e:
        short.take_sgt(0, sims[0][0])
    assert e.value.code == 6


@pytest.mark.parametrize("mode", [1, 2])
def test_filtered_kernels_bitwise(mode, oracle_mod, native_lib):
    """Filtering of the synthetics and of the two series before the window integral
    (SI_ker_sta.F90:756-773; filter / filtfilt :1433-1558): the device filter of every
    point's series and the host filter of V, U equal the restatement bit for bit."""
    import fwant_gb300 as fw
    signal = pytest.importorskip("scipy.signal")
    b, a = signal.butter(3, [0.04, 0.3], btype="band")  # 7 coefficients: 18 padding samples
    rng = np.random.default_rng(40 + mode)
    npts, knt, dt, nt1, nt2 = 131, 300, 0.1, 21, 280  # 131 points: a partial block of 128
    lam, mu = _media(rng, npts)
    r = [_series(rng, npts, knt) for _ in range(3)]
    s = _series(rng, npts, knt)
    k = fw.SgtKernel(npts, knt, dt)
    k.set_media(lam, mu)
    for c in range(3):
        k.set_sgt(c, r[c])
    k.set_sgt(3, s)
    k.scatter(7)
    scat = oracle_mod.sgt2scatter3(lam, mu, r, s, dt, mode=1)
    v = rng.normal(size=knt).astype(np.float32)
    u = np.cumsum(v).astype(np.float32) * np.float32(dt)
    for ncmp, (sa, sb) in ((1, (0, 3)), (2, (1, 5)), (3, (2, 4))):
        got = k.kernel(ncmp, v, u, nt1, nt2, 1.0e16, filt=(mode, b, a))
        want = oracle_mod.scatter2kernel_filtered(v, u, scat[sa], scat[sb], dt, nt1, nt2, 1.0e16, b, a, mode)
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w)
        plain = k.kernel(ncmp, v, u, nt1, nt2, 1.0e16)
        assert not np.allclose(plain[0], got[0], rtol=1e-3, atol=0.0)  # the filter changed the kernel
    # the unfiltered series are kept: a plain call after a filtered one is unchanged
    np.testing.assert_array_equal(k.kernel(1, v, u, nt1, nt2, 1.0e16)[0],
                                  oracle_mod.scatter2kernel(v, u, scat[0], scat[3], dt, nt1, nt2, 1.0e16, mode=1)[0])
    for bad in ((3, b, a), (1, np.ones(17), np.ones(17)), (1, b, np.r_[0.0, a[1:]])):
        with pytest.raises(fw.FwantError) as e:
            k.kernel(1, v, u, nt1, nt2, 1.0e16, filt=bad)
        assert e.value.code == 1
    short = fw.SgtKernel(npts, 18, dt)  # 18 frames: not more than the 18 padding samples
    short.set_media(lam, mu)
    for c in range(4):
        short.set_sgt(c if c < 3 else 3, np.ascontiguousarray((r[c] if c < 3 else s)[:, :18]))
    short.scatter(1)
    with pytest.raises(fw.FwantError) as e:
        short.kernel(1, v[:18], u[:18], 1, 18, 1.0e16, filt=(mode, b, a))
    assert e.value.code == 1


def test_rotation_of_the_force_components(oracle_mod, native_lib):
    """scatter_rotate (SI_ker_sta.F90:1357-1373): the three force components' series mixed
    by the rotation matrix, rot(d, c) weighting component d into c, summed in order."""
    import fwant_gb300 as fw
    rng = np.random.default_rng(77)
    npts, knt, dt = 40, 90, 0.2
    lam, mu = _media(rng, npts)
    r = [_series(rng, npts, knt) for _ in range(3)]
    s = _series(rng, npts, knt)
    k = fw.SgtKernel(npts, knt, dt)
    k.set_media(lam, mu)
    for c in range(3):
        k.set_sgt(c, r[c])
    k.set_sgt(3, s)
    k.scatter(3)
    with pytest.raises(fw.FwantError) as e:
        k.rotate(np.eye(3))  # Z not computed
    assert e.value.code == 6
    k.scatter(7)
    th = 0.7
    rot = np.array([[np.cos(th), np.sin(th), 0.0], [-np.sin(th), np.cos(th), 0.0], [0.0, 0.0, 1.0]])
    rot = rot @ np.array([[1.0, 0.0, 0.0], [0.0, np.cos(0.3), -np.sin(0.3)], [0.0, np.sin(0.3), np.cos(0.3)]])
    before = [k.get_scatter(q) for q in range(6)]
    k.rotate(rot)
    for group in ((0, 1, 2), (3, 5, 4)):
        v = [before[q] for q in group]
        for c in range(3):
            want = (v[0] * rot[0, c] + v[1] * rot[1, c]) + v[2] * rot[2, c]
            np.testing.assert_array_equal(k.get_scatter(group[c]), want)


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_parameter_conversion_bitwise(mode, native_lib):
    """fwant_sgtker_convert (SI_ker_lamu2kamu / SI_ker_lamu2vpvs / SI_ker_vpvs2kamu) equals the
    single-precision restatement bit for bit on random kernels and media; a mode outside 1..3
    is refused."""
    import fwant_gb300 as fw
    from oracle import kconv_oracle as KC
    rng = np.random.default_rng(40 + mode)
    n = 5000
    vp = rng.uniform(5.5e3, 8.0e3, n)
    vs = vp / rng.uniform(1.65, 1.85, n)
    rho = rng.uniform(2.5e3, 3.3e3, n)
    mu = (rho * vs * vs).astype(np.float32)
    lam = (rho * vp * vp - 2 * rho * vs * vs).astype(np.float32)
    kern = [(rng.normal(size=n) * 1e-9).astype(np.float32) for _ in range(4)]
    k = fw.SgtKernel(n, 4, 0.1)
    k.set_media(lam, mu)
    got = k.convert(mode, *kern)
    for ph in (0, 1):
        a, b = KC.convert(mode, lam, mu, kern[ph], kern[2 + ph])
        np.testing.assert_array_equal(got[ph], a)
        np.testing.assert_array_equal(got[2 + ph], b)
    with pytest.raises(Exception):
        k.convert(4, *kern)
    k.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_pair_bitwise_against_the_restatement(mode, native_lib):
    """SI_ker_pair on the device: the single-precision scatter series of one receiver SGT
    against the source SGT, and the window kernels after each filter mode, equal the
    restatement (oracle/kpair_oracle.py) bit for bit; lags across several staging chunks
    (knt 700)."""
    import fwant_gb300 as fw
    from oracle import kpair_oracle as KP
    signal = pytest.importorskip("scipy.signal")
    rng = np.random.default_rng(31 + mode)
    npts, knt, dt = 29, 700 if mode == 0 else 160, np.float32(0.1)
    lam, mu = _media(rng, npts)
    rs, ss = _series(rng, npts, knt), _series(rng, npts, knt)
    K = fw.SgtKernel(npts, knt, float(dt))
    K.set_media(lam, mu)
    K.set_sgt(0, rs)
    K.set_sgt(3, ss)
    K.scatter_pair()
    sa, sb = KP.scatter_pair(lam, mu, rs, ss, float(dt))
    np.testing.assert_array_equal(K.get_scatter(0), sa)
    np.testing.assert_array_equal(K.get_scatter(1), sb)
    b, a = signal.butter(2, [0.05, 0.3], btype="band")
    v = rng.normal(size=knt).astype(np.float32)
    u = np.cumsum(v).astype(np.float32) * dt
    for nt1, nt2 in ((1, knt), (7, knt // 2), (knt // 3, knt - 5)):
        got = K.kernel_pair(v, u, nt1, nt2, 1.0e15, mode=mode, b=b, a=a)
        want = KP.kernel_pair(v, u, sa, sb, float(dt), nt1, nt2, 1.0e15, mode=mode, b=b, a=a)
        for q in range(4):
            np.testing.assert_array_equal(got[q], np.asarray(want[q]).astype(np.float32), err_msg=f"{nt1} {nt2} {q}")
            assert np.any(got[q])
    with pytest.raises(fw.FwantError):
        K.kernel_pair(v, u, 0, knt, 1.0e15)
    # a scatter of SI_ker_sta replaces the pair's series: the pair kernel is refused after it
    K.scatter(1)
    with pytest.raises(fw.FwantError):
        K.kernel_pair(v, u, 1, knt, 1.0e15)
    K.close()
