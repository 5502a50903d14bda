"""Physics checks of the oracle (the CPU restatement of seis3d_wave) that a restatement
error could not pass by construction: source-receiver reciprocity of surface forces,
energy decay once the wavefield has entered the CFS-PML, and convergence under grid
refinement.  The same experiments run on the GPU in test_gpu_physics.py.

Measured on the oracle (FP32, seeded models of tests/physics.py):
* reciprocity G_ij(A <- B) = G_ji(B <- A): the diagonal and the two horizontal cross
  pairs agree within 0.1-0.4%; the horizontal-vertical cross pairs carry a first-order
  discretisation asymmetry of the surface traction source and free surface (13-15% at a
  1 km surface spacing, 4.5-6.8% at 0.5 km, 2.6-5.9% at 0.25 km) with the same waveform
  (correlation > 0.999);
* energy outside the PML decays monotonically after the source stops, by nine orders of
  magnitude in 1200 steps, against five without a PML (the zero ghost values reflect);
* an isotropic stress pulse (4 km Gaussian) in a homogeneous 48 km cube: successive
  differences 3.7e-4 and 6.0e-5 at 1, 0.5 and 0.25 km, an observed order of 2.6 at these
  (4 to 16 cells per pulse width) resolutions, rising towards the scheme's fourth order
  with a finer level on the GPU;
* a pure P pulse (isotropic stress) and a pure S pulse (rotational velocity) in a
  homogeneous cube against the closed-form solutions of the wave equation at Vp and Vs
  along a line through the centre: 1.8% / 2.2% relative L2 at 1 km spacing, 0.17% / 0.17%
  at 0.5 km (a 1% error in either speed would move the pulse 140 m and cost ~7%);
* the Rayleigh pulse of a vertical surface force on a homogeneous half-space travels at
  the half-space's Rayleigh speed (0.919 Vs): 1.4% slow at 0.5 km spacing, 0.35% at
  0.25 km (measured on the oracle; a surface without the traction condition has no such
  wave)."""
import numpy as np
import pytest

import physics as P


def _make(O):
    return lambda ni, nj, nk, stept, fs: O.Oracle(ni, nj, nk, stept, free_surface=fs)


def test_reciprocity_of_surface_forces(oracle_mod):
    oracle_mod.set_threads(0)
    errs = {}
    for top, bottom, nk in ((1.0, 1.0, 24), (0.5, 2.0, 28)):
        m, a, b, nsteps = P.reciprocity_model(z_top_km=top, z_bottom_km=bottom, nk=nk)
        g = P.reciprocity_gathers(_make(oracle_mod), m, a, b, nsteps)
        errs[top] = P.reciprocity_errors(g, a, b)
        print(top, {k: round(v, 4) for k, v in errs[top].items()})
    fine, coarse = errs[0.5], errs[1.0]
    same_plane = [("x", "x"), ("y", "y"), ("z", "z"), ("x", "y"), ("y", "x")]
    for k in same_plane:
        assert fine[k] < 0.01, (k, fine[k])
        assert coarse[k] < 0.02, (k, coarse[k])
    for k in (("x", "z"), ("z", "x"), ("y", "z"), ("z", "y")):
        assert fine[k] < 0.10, (k, fine[k])
        # the surface asymmetry shrinks with the surface spacing (first order)
        assert coarse[k] > 1.6 * fine[k], (k, coarse[k], fine[k])


def test_energy_decays_in_the_pml(oracle_mod):
    oracle_mod.set_threads(0)
    out = {}
    for npml in (8, 0):
        m = P.energy_model(npml)
        t, e = P.energy_history(_make(oracle_mod), m, 10, 1200, 20)
        out[npml] = e / e.max()
    e = out[8]
    peak = int(np.argmax(e))
    after = e[peak:]
    assert np.all(after[1:] <= after[:-1] * (1 + 1e-3)), after
    assert after[-1] < 1e-7
    # the reflecting boundary keeps orders of magnitude more energy in the model
    assert out[0][-1] > 100 * after[-1]
    assert np.any(np.diff(out[0][peak:]) > 0)


def test_convergence_under_refinement(oracle_mod):
    oracle_mod.set_threads(0)
    sols = [P.convergence_solution(_make(oracle_mod), level) for level in range(3)]
    errs, orders = P.convergence_orders(sols)
    print("differences", errs, "orders", orders)
    assert errs[0] < 1e-3 and errs[1] < errs[0]
    assert orders[0] > 2.3


@pytest.mark.parametrize("kind", ["P", "S"])
def test_pulses_travel_at_the_medium_speeds(kind, oracle_mod):
    oracle_mod.set_threads(0)
    errs = []
    for level in (0, 1):
        d, num, exact = P.pulse_line(_make(oracle_mod), kind, level=level)
        errs.append(float(np.linalg.norm(num - exact) / np.linalg.norm(exact)))
    print(kind, errs)
    assert errs[0] < 0.03 and errs[1] < 0.004 and errs[1] < errs[0] / 5, errs


def test_rayleigh_wave_speed(oracle_mod):
    oracle_mod.set_threads(0)
    c, cr = P.rayleigh_speed(_make(oracle_mod), 0.5)
    print(c, cr, c / cr - 1)
    assert abs(c / cr - 1) < 0.025, (c, cr)


@pytest.mark.parametrize("kind", ["P", "S"])
def test_pulse_check_detects_a_one_percent_speed_error(kind, oracle_mod):
    """The pulse check has teeth: the oracle given lambda and mu 2.01% too large (wave
    speeds 1% too fast) lands at 8.9% (P) / 6.4% (S) from the closed form at 1 km spacing,
    against 1.8% / 2.2% with the true medium."""
    oracle_mod.set_threads(0)

    def make(ni, nj, nk, stept, fs):
        s = oracle_mod.Oracle(ni, nj, nk, stept, free_surface=fs)
        set_media = s.set_media
        s.set_media = lambda lam, mu, rho: set_media(lam * np.float32(1.0201), mu * np.float32(1.0201), rho)
        return s

    d, num, exact = P.pulse_line(make, kind, level=0)
    assert np.linalg.norm(num - exact) / np.linalg.norm(exact) > 0.05
