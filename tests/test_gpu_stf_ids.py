"""Every source time function id on the GPU path against the oracle
(src_stf / src_svf, code/srcF/mod_src.F90:438-622).

Which function a source reads depends on its kind, as in the reference:
* a surface force under a free surface (src_surface, :373-414) reads both src_stf (the
  traction image) and src_svf (the velocity boundary term), so only ids defined by both
  run (220, 200, 230, 100, 240); 250, 120 and 110 stop the run on both sides;
* a body force without a free surface (src_force, :275-345) reads src_stf alone, so
  the delta id 250 runs there;
* a moment tensor (src_stress, :207-273) reads src_svf alone: 120 and 110 run, 250 does
  not.
Exact form: per field and seismogram component within 1e-6 relative L2 (bit-identical in
practice); fast form within 1e-5."""
import numpy as np
import pytest

from helpers import MOMENT, interior, rel_l2, small_model

pytestmark = pytest.mark.gpu

# (window start t0 = stf_time, frequency or rise time f0 = stf_freq) per family, chosen so
# that the function is active over the 24 steps (about 0.75 s) of the run
WINDOW = {200: (0.6, 2.0), 220: (0.4, 0.2), 120: (0.4, 0.2), 230: (0.05, 0.5), 100: (0.05, 0.5),
          110: (0.05, 0.5), 240: (0.0, 1.0), 250: (0.0, 1.0)}
CASES = ([("surface", i, True) for i in (220, 200, 230, 100, 240)] +
         [("surface", i, False) for i in (250, 120, 110)] +
         [("nofree", i, True) for i in (220, 200, 230, 100, 240, 250)] +
         [("nofree", i, False) for i in (120, 110)] +
         [("moment", i, True) for i in (120, 220, 200, 100, 230, 110, 240)] +
         [("moment", 250, False)])


def _feed(s, m, met, kind, stf_id):
    t0, f0 = WINDOW[stf_id]
    s.set_coord(m.x, m.y, m.z)
    s.set_metric(met["xsin"], met["xcot"], met["xi_x"], met["eta_y"], met["zeta_z"])
    s.set_media(m.lam, m.mu, m.rho)
    s.set_pml(m.pml_number, m.pml_velocity, m.pml_bmax, m.pml_amax)
    if kind == "moment":
        s.set_moments(m.force_indx, m.force_shift, m.force_t0, [t0], [f0], MOMENT["mom"], stf_id)
    else:
        s.set_forces(m.force_indx, m.force_shift, m.force_t0, [t0], [f0], m.fx, m.fy, m.fz, stf_id)
    s.set_receivers(m.recv_indx, m.recv_tinv)
    return s


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
@pytest.mark.parametrize("kind,stf_id,runs", CASES, ids=[f"{k}-{i}" for k, i, _ in CASES])
def test_stf_id_against_oracle(kind, stf_id, runs, exact, oracle_mod, native_lib):
    import fwant_gb300 as fw
    m = small_model("moment" if kind == "moment" else kind)
    met = oracle_mod.metric(m.x, m.y, m.z)
    g = _feed(fw.Solver(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface, exact_arith=exact), m, met, kind,
              stf_id)
    o = _feed(oracle_mod.Oracle(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface), m, met, kind, stf_id)
    if not runs:
        with pytest.raises(RuntimeError, match="unknown"):
            o.run(8)
        with pytest.raises(fw.FwantError) as e:
            g.run(8)
        assert e.value.code == 1
        return
    g.run(24)
    o.run(24)
    tol = 1e-6 if exact else 1e-5
    live = 0
    for c in range(9):
        a, b = interior(g.get_field(c)), interior(o.get_field(c))
        if not np.any(b):
            assert not np.any(a), f"component {c}: expected zeros"
            continue
        live += 1
        assert rel_l2(a, b) < tol, f"component {c}: {rel_l2(a, b):.3e}"
    assert live > 0, "the source never acted"
    # Seismogram errors relative to the norm of their group (velocities, stresses): the
    # free-surface condition holds Tzz, Txz and Tyz of surface receivers at rounding level
    # away from the source, and a component-wise ratio of two rounding residues says nothing.
    sg, so = g.get_seismo().astype(np.float64), o.get_seismo()
    assert sg.shape == so.shape
    for grp in (slice(0, 3), slice(3, 9)):
        den = np.sqrt(np.sum(so[grp] ** 2))
        for c in range(grp.start, grp.stop):
            e = np.sqrt(np.sum((sg[c] - so[c]) ** 2)) / den
            assert e < tol, f"seismogram {c}: {e:.3e} of its group's norm"
