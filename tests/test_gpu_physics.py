"""The physics checks of test_physics_oracle.py on the GPU's fast arithmetic form, with
finer levels than the CPU can afford: the reciprocity asymmetry of the horizontal-vertical
pairs must keep shrinking at a 0.25 km surface spacing, and the convergence study adds a
0.125 km level (385^3 points), where the observed order reaches 3.7 (successive
differences 3.7e-4, 6.0e-5, 4.7e-6).  The P and S pulses of the oracle test, against
their closed-form solutions, add a 0.25 km level: P 1.8%, 0.17%, 0.015%; S 2.2%, 0.17%,
0.021% at 1, 0.5 and 0.25 km (an observed order of 3.2-3.5).  The Rayleigh pulse of the
oracle test runs at 0.5, 0.25 and 0.125 km spacing and must approach the half-space's
Rayleigh speed: 1.43%, 0.36% and 0.24% slow."""
import numpy as np
import pytest

import physics as P

pytestmark = pytest.mark.gpu


def _make():
    import fwant_gb300 as fw
    return lambda ni, nj, nk, stept, fs: fw.Solver(ni, nj, nk, stept, free_surface=fs)


def test_reciprocity_of_surface_forces_gpu(native_lib):
    errs = {}
    for top, bottom, nk in ((1.0, 1.0, 24), (0.5, 2.0, 28), (0.25, 2.0, 36)):
        m, a, b, nsteps = P.reciprocity_model(z_top_km=top, z_bottom_km=bottom, nk=nk)
        g = P.reciprocity_gathers(_make(), m, a, b, nsteps)
        errs[top] = P.reciprocity_errors(g, a, b)
        print(top, {k: round(v, 4) for k, v in errs[top].items()})
    for k in (("x", "x"), ("y", "y"), ("z", "z"), ("x", "y"), ("y", "x")):
        assert errs[0.5][k] < 0.01 and errs[0.25][k] < 0.01, k
    for k in (("x", "z"), ("z", "x"), ("y", "z"), ("z", "y")):
        assert errs[0.5][k] < 0.10, k
        assert errs[1.0][k] > 1.6 * errs[0.5][k], k
        assert errs[0.25][k] < errs[0.5][k], k


def test_energy_decays_in_the_pml_gpu(native_lib):
    out = {}
    for npml in (8, 0):
        m = P.energy_model(npml)
        _, e = P.energy_history(_make(), m, 10, 1200, 20)
        out[npml] = e / e.max()
    e = out[8]
    peak = int(np.argmax(e))
    after = e[peak:]
    assert np.all(after[1:] <= after[:-1] * (1 + 1e-3)), after
    assert after[-1] < 1e-7
    assert out[0][-1] > 100 * after[-1]


def test_convergence_under_refinement_gpu(native_lib):
    sols = [P.convergence_solution(_make(), level) for level in range(4)]
    errs, orders = P.convergence_orders(sols)
    print("differences", errs, "orders", orders)
    assert all(errs[l + 1] < errs[l] for l in range(len(errs) - 1))
    assert orders[0] > 2.3 and orders[1] > 3.3


@pytest.mark.parametrize("kind", ["P", "S"])
def test_pulses_travel_at_the_medium_speeds_gpu(kind, native_lib):
    errs = []
    for level in (0, 1, 2):
        d, num, exact = P.pulse_line(_make(), kind, level=level)
        errs.append(float(np.linalg.norm(num - exact) / np.linalg.norm(exact)))
    print(kind, errs)
    assert errs[0] < 0.03 and errs[1] < 0.004 and errs[1] < errs[0] / 5, errs
    assert errs[2] < errs[1], errs


def test_rayleigh_wave_speed_gpu(native_lib):
    errs = []
    for dh in (0.5, 0.25, 0.125):
        c, cr = P.rayleigh_speed(_make(), dh)
        errs.append(c / cr - 1)
    print(errs)
    assert abs(errs[0]) < 0.025 and abs(errs[1]) < 0.006, errs
    assert abs(errs[2]) < abs(errs[1]), errs
