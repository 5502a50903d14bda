"""The terrain-following grid on the GPU (the Gaussian-hill extension; no counterpart in
the reference, whose grid is orthogonal spherical with a flat top):

* a zero hill reproduces today's flat solver bit for bit in the reference-order form, and
  within FP32 rounding in the fast form (the two kernel instantiations contract FMAs
  independently);
* the device's FP64 terrain metric equals the FP32 oracle's bit for bit;
* on a 2 km hill the GPU agrees with the FP32 oracle within 1e-5 and with the FP64 oracle
  within 1e-4 relative L2 (fields on the planes k <= nk2 and seismograms; above the free
  surface the oracle stores its image values and the GPU, which substitutes images while
  loading, stores none);
* self-convergence on the hill: seismograms at 1 to 0.125 km spacing (same physical model)
  converge, the finest halving shrinking the difference by more than 2x, no worse than the
  flat top's."""
import numpy as np
import pytest

from topo_case import LENFD, convergence_level, hill_model, rel

pytestmark = pytest.mark.gpu

KINDS = ("surface", "buried")


def _solver(m, exact, metric):
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    return inputs.attach(fw.Solver(m.ni, m.nj, m.nk, m.stept, exact_arith=exact), m, metric=metric)


@pytest.mark.parametrize("kind", KINDS)
def test_zero_hill_is_the_flat_solver(kind, oracle_mod, native_lib):
    m, h = hill_model(kind=kind)
    met = oracle_mod.metric(m.x, m.y, m.z)
    for exact in (True, False):
        flat = _solver(m, exact, met)
        zero = _solver(m, exact, met)
        zero.set_topography(np.zeros_like(h))
        flat.run(24)
        zero.run(24)
        for c in range(9):
            a, b = zero.get_field(c), flat.get_field(c)
            if exact:
                assert np.array_equal(a, b), f"{kind} component {c}: {int(np.sum(a != b))} values differ"
            else:
                assert rel(a, b) < 1e-6, (kind, c, rel(a, b))
        sa, sb = zero.get_seismo(), flat.get_seismo()
        if exact:
            assert np.array_equal(sa, sb)
        else:
            assert rel(sa, sb) < 1e-6
        flat.close()
        zero.close()


def test_terrain_metric_equals_the_oracle(oracle_mod, native_lib):
    from fwant_gb300 import inputs
    m, h = hill_model()
    met = oracle_mod.metric(m.x, m.y, m.z)
    g = _solver(m, False, met)
    g.set_topography(h)
    o = oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept)
    inputs.attach(o, m, metric=met)
    o.set_topography(h)
    for w in range(7):
        a, b = g.topography_array(w), o.topography_array(w).astype(np.float32)
        assert np.array_equal(a, b), f"array {w}: {int(np.sum(a != b))} values differ"
    g.close()


@pytest.mark.parametrize("kind", KINDS)
def test_hill_against_the_oracle(kind, oracle_mod, native_lib):
    from fwant_gb300 import inputs
    m, h = hill_model(kind=kind)
    met = oracle_mod.metric(m.x, m.y, m.z)
    steps = 300
    refs = {}
    for dbl in (False, True):
        o = oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept, dbl=dbl)
        inputs.attach(o, m, metric=met)
        o.set_topography(h)
        o.run(steps)
        refs[dbl] = ([o.get_field(c) for c in range(9)], o.get_seismo())
    for exact in (True, False):
        g = _solver(m, exact, met)
        g.set_topography(h)
        g.run(steps)
        fields = [g.get_field(c) for c in range(9)]
        sg = g.get_seismo()
        g.close()
        k2 = LENFD + m.nk - 1
        for dbl, tol in ((False, 1e-5), (True, 1e-4)):
            rf, rs = refs[dbl]
            worst = max(rel(fields[c][:, :, :k2 + 1], rf[c][:, :, :k2 + 1]) for c in range(9))
            assert worst < tol, (kind, exact, dbl, worst)
            assert rel(sg[:3], rs[:3]) < tol and rel(sg[3:], rs[3:]) < tol, (kind, exact, dbl)


def _convergence_traces(amp, levels):
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    traces = []
    for level in range(levels):
        m, h = convergence_level(level, amp=amp)
        s = inputs.attach(fw.Solver(m.ni, m.nj, m.nk, m.stept), m)
        s.set_topography(h)
        s.run(int(round(24.0 / 0.05)) * 2 ** level)
        sg = s.get_seismo()[:3].astype(np.float64)   # velocities (3, nsamp, 4)
        traces.append(sg[:, 2 ** level - 1::2 ** level, :])   # samples at level-0 times
        s.close()
    n = min(t.shape[1] for t in traces)
    traces = [t[:, :n, :] for t in traces]
    ref = np.sqrt(np.sum(traces[-1] ** 2))
    assert np.all(np.isfinite(traces[-1])) and ref > 0
    return [float(np.sqrt(np.sum((traces[l] - traces[l + 1]) ** 2)) / ref) for l in range(levels - 1)]


def test_hill_self_convergence(native_lib):
    """Seismograms of a force 6 km under the hill top at 1, 0.5, 0.25 and 0.125 km spacing
    (the same physical model at every level): successive differences shrink, by more than
    2x at the finest halving, and stay within 2x of the flat top's (h = 0) at each level."""
    flat = _convergence_traces(0.0, 4)
    hill = _convergence_traces(2000.0, 4)
    print("self-convergence differences: flat", flat, "hill", hill,
          "hill orders", [np.log2(hill[l] / hill[l + 1]) for l in range(len(hill) - 1)])
    assert all(hill[l + 1] < hill[l] for l in range(len(hill) - 1))
    assert hill[-1] < hill[-2] / 2.0
    assert all(hill[l] < 2.0 * flat[l] for l in range(len(hill)))
