"""Reduced-precision storage of the wavefield registers (BF16 and FP16, FP32 arithmetic).

The FP32 CPU restatement is the reference.  Each storage kind is held to the error its
rounding predicts over a 75-step run (relative L2 of the interior fields and of the
seismograms).  BF16 keeps 8 significant bits (unit roundoff u = 2^-8 = 3.9e-3), FP16 keeps
11 (u = 2^-11 = 4.9e-4) once power-of-two scales bring the field into its normal range.
Every step rounds four stage outputs; the wave equation neither damps nor amplifies the
rounding noise much, so it adds up like a random walk: after n steps the relative error is
about sqrt(4 n) * u / sqrt(3) (the RMS of a uniform rounding error is u / sqrt(3)), i.e.
3.9e-2 (BF16) and 4.9e-3 (FP16) for n = 75.  The bounds below are three times that.
"""
import numpy as np
import pytest

from helpers import feed, interior, rel_l2, small_model

pytestmark = pytest.mark.gpu

NSTEPS = 75
STORAGE_TOL = {k: 3.0 * np.sqrt(4 * NSTEPS) * u / np.sqrt(3.0) for k, u in (("bf16", 2.0 ** -8), ("fp16", 2.0 ** -11))}


def _storage_id(name):
    import fwant_gb300 as fw
    return {"fp32": fw.STORAGE_FP32, "bf16": fw.STORAGE_BF16, "fp16": fw.STORAGE_FP16}[name]


def _solver(m, met, kind, storage, scales=None):
    import fwant_gb300 as fw
    s = fw.Solver(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface, storage=_storage_id(storage))
    if scales is not None:
        s.set_storage_scale(*scales)
    return feed(s, m, met, kind)


def _peak_max_abs(m, met, kind, nsteps, every=5):
    """Per-component max |value| over the whole run of an FP32 solve (sampled every few
    steps: near-source peaks pass long before the end of the run)."""
    probe = _solver(m, met, kind, "fp32")
    mx = np.zeros(9, np.float32)
    done = 0
    while done < nsteps:
        n = min(every, nsteps - done)
        probe.run(n)
        done += n
        mx = np.maximum(mx, probe.max_abs())
    return mx, probe


def _scales(maxabs):
    """Powers of two that put the largest velocity and stress near 2^13 (FP16 headroom 8x)."""
    v = float(np.max(maxabs[:3]))
    t = float(np.max(maxabs[3:]))
    return tuple(float(2.0 ** np.floor(np.log2(8192.0 / x))) if x > 0 else 1.0 for x in (v, t))


@pytest.mark.parametrize("storage", ["bf16", "fp16"])
@pytest.mark.parametrize("kind", ["surface", "buried", "nofree"])
def test_reduced_storage_against_fp32_oracle(kind, storage, oracle_mod, native_lib):
    m = small_model(kind)
    met = oracle_mod.metric(m.x, m.y, m.z)
    o = feed(oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface), m, met, kind)
    o.run(NSTEPS)
    scales = None
    if storage == "fp16":
        scales = _scales(_peak_max_abs(m, met, kind, NSTEPS)[0])
    g = _solver(m, met, kind, storage, scales)
    g.run(40)
    g.run(NSTEPS - 40)
    g.check()
    errs = {}
    for c in range(9):
        a, b = interior(g.get_field(c)), interior(o.get_field(c))
        if np.any(b):
            errs[f"field {c}"] = rel_l2(a, b)
    sg, so = g.get_seismo(), o.get_seismo()
    for c in range(9):
        if np.any(so[c]):
            errs[f"seismogram {c}"] = rel_l2(sg[c], so[c])
    print(f"{kind}/{storage}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    worst = max(errs, key=errs.get)
    assert errs[worst] < STORAGE_TOL[storage], f"{kind}/{storage} {worst}: {errs[worst]:.3e}"


def test_fp16_without_scaling_overflows(oracle_mod, native_lib):
    """Stresses of ~3e6 Pa exceed FP16's 65504: unscaled FP16 storage turns them into Inf,
    which the overflow check reports; the scaled run keeps them.  Guards that the scale
    is applied on every store and load."""
    import fwant_gb300 as fw
    m = small_model("buried")
    met = oracle_mod.metric(m.x, m.y, m.z)
    mx, probe = _peak_max_abs(m, met, "buried", 40)
    assert np.max(mx[3:]) > 65504.0, "test premise: stresses above FP16's range"
    scaled = _solver(m, met, "buried", "fp16", _scales(mx))
    scaled.run(40)
    scaled.check()
    assert rel_l2(interior(scaled.get_field("Tzz")), interior(probe.get_field("Tzz"))) < STORAGE_TOL["fp16"]
    plain = _solver(m, met, "buried", "fp16")
    plain.run(40)
    with pytest.raises(fw.FwantError) as e:
        plain.check()
    assert e.value.code == 4


def test_max_abs_matches_fields(oracle_mod, native_lib):
    import fwant_gb300 as fw
    m = small_model("moment")
    met = oracle_mod.metric(m.x, m.y, m.z)
    g = feed(fw.Solver(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface, exact_arith=True), m, met, "moment")
    g.run(20)
    mx = g.max_abs()
    want = np.array([np.max(np.abs(g.get_field(c))) for c in range(9)], np.float32)
    np.testing.assert_array_equal(mx, want)


@pytest.mark.parametrize("storage", ["bf16", "fp16"])
def test_field_round_trip_in_reduced_storage(storage, native_lib):
    """set_field then get_field: values representable in the storage type (after scaling)
    come back exactly; others come back rounded to nearest."""
    import fwant_gb300 as fw
    m = small_model("surface")
    s = fw.Solver(m.ni, m.nj, m.nk, m.stept, storage=_storage_id(storage))
    s.set_storage_scale(2.0 ** 10, 2.0 ** -20)
    rng = np.random.default_rng(5)
    v = np.zeros(s.shape, np.float32)
    t = np.zeros(s.shape, np.float32)
    sl = (slice(3, -3),) * 3
    # integers up to 255 are exact in both kinds; divide by the scale
    v[sl] = rng.integers(-255, 256, size=v[sl].shape).astype(np.float32) / np.float32(2.0 ** 10)
    t[sl] = rng.integers(-255, 256, size=t[sl].shape).astype(np.float32) * np.float32(2.0 ** 20)
    s.set_field("Vy", v)
    s.set_field("Txz", t)
    np.testing.assert_array_equal(s.get_field("Vy"), v)
    np.testing.assert_array_equal(s.get_field("Txz"), t)
    # a value between two representable ones rounds to nearest
    x = np.zeros(s.shape, np.float32)
    x[10, 10, 10] = np.float32(1.0 + 2.0 ** -15) / np.float32(2.0 ** 10)
    s.set_field("Vx", x)
    assert s.get_field("Vx")[10, 10, 10] == np.float32(1.0 / 2.0 ** 10)
    mx = s.max_abs()
    assert mx[1] == np.max(np.abs(v)) and mx[7] == np.max(np.abs(t))


def test_storage_scale_rules(native_lib):
    import fwant_gb300 as fw
    m = small_model("surface")
    s = fw.Solver(m.ni, m.nj, m.nk, m.stept, storage=fw.STORAGE_FP16)
    with pytest.raises(fw.FwantError) as e:
        s.set_storage_scale(3.0, 1.0)
    assert e.value.code == 1
    with pytest.raises(fw.FwantError):
        s.set_storage_scale(0.0, 1.0)
    from fwant_gb300 import inputs
    inputs.attach(s, m)
    s.set_storage_scale(4.0, 0.25)
    s.run(1)
    with pytest.raises(fw.FwantError) as e:
        s.set_storage_scale(1.0, 1.0)
    assert e.value.code == 6
    with pytest.raises(fw.FwantError) as e:
        fw.Solver(m.ni, m.nj, m.nk, m.stept, storage=fw.STORAGE_FP64)
    assert e.value.code == 1
    with pytest.raises(fw.FwantError) as e:
        fw.Solver(m.ni, m.nj, m.nk, m.stept, storage=fw.STORAGE_BF16, exact_arith=True)
    assert e.value.code == 1


def test_bf16_run_is_deterministic(oracle_mod, native_lib):
    m = small_model("buried")
    met = oracle_mod.metric(m.x, m.y, m.z)
    a = _solver(m, met, "buried", "bf16")
    b = _solver(m, met, "buried", "bf16")
    a.run(24)
    b.run(16)
    b.run(8)
    for c in range(9):
        np.testing.assert_array_equal(a.get_field(c), b.get_field(c))
    np.testing.assert_array_equal(a.get_seismo(), b.get_seismo())
