"""Configuration files of the input preprocessors (SeisFD3D.conf with its grid, source and
station keys, the grid and source configurations) and the fwant_prep runner, shared by the
fwant_prep tests."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_prep")
NI, NJ, NK = 20, 16, 12


def f32text(v) -> str:
    """text that reads back as the same float32 value"""
    return repr(float(np.float32(v)))


def write(path, lines):
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main_conf(tmp, extra=(), ni=NI, nj=NJ, nk=NK):
    path = os.path.join(tmp, "SeisFD3D.conf")
    write(path, [f"ni = {ni}", f"nj = {nj}", f"nk = {nk}", "nt = 10", "stept = 0.01", "dims = 1 1 1",
                  f"GRID_CONF = {tmp}/SeisGrid.conf   # grid generation", f"GRID_ROOT = {tmp}",
                  f"SOURCE_CONF = {tmp}/SeisSource.conf", f"SOURCE_ROOT = {tmp}", f"STATION_ROOT = {tmp}",
                  *extra])
    return path


def grid_conf(tmp, steph=(0.009, 0.009, 0.5), origin=(45.5, 100.0, 6371.0), d2m=1000.0, lists=()):
    lines = ["# grid of the tests", f"distance2meter = {f32text(d2m)}",
             "steph = " + " ".join(f32text(v) for v in steph) + "   # degree degree km",
             "theta0_phi0_rmax | " + " ".join(f32text(v) for v in origin)]
    for anchor, vals in lists:
        lines.append(f"{anchor}    # list of values")
        for q in range(0, len(vals), 5):   # five values a line, comma separated
            lines.append(", ".join(f32text(v) for v in vals[q:q + 5]))
    write(os.path.join(tmp, "SeisGrid.conf"), lines)


def run(stage, conf, ok=True):
    r = subprocess.run([EXE, stage, conf], capture_output=True, text=True)
    if ok:
        assert r.returncode == 0, r.stdout + r.stderr
    return r


def read(path):
    from scipy.io import netcdf_file
    with netcdf_file(path, "r", mmap=False) as f:
        return {k: np.array(v[:]) for k, v in f.variables.items()}, dict(f._attributes), dict(f.dimensions)


def source_conf(tmp, hyper, forces, ntw_f, moments, ntw_m, mech, stf_f="ricker", stf_m="gauss"):
    lines = [f"src_hyper_height = {f32text(hyper)}", f"number_of_force_source = {len(forces) // max(ntw_f, 1)}"]
    if forces:
        lines += [f"force_stf_window = {ntw_f}", f"force_stf_type = {stf_f}",
                  "force_stf_timefactor = " + " ".join(f32text(1.5 + q) for q in range(ntw_f)),
                  "force_stf_freqfactor = " + " ".join(f32text(0.25 * (q + 1)) for q in range(ntw_f))]
    lines.append(f"number_of_moment_source = {len(moments) // max(ntw_m, 1)}")
    if moments:
        lines += [f"moment_stf_window = {ntw_m}", f"moment_stf_type = {stf_m}",
                  "moment_stf_timefactor = " + " ".join(f32text(2.0 + q) for q in range(ntw_m)),
                  "moment_stf_freqfactor = " + " ".join(f32text(0.5 * (q + 1)) for q in range(ntw_m)),
                  f"moment_mech_input = {mech}"]
    lines.append("<anchor_force>")
    for r in forces:
        lines.append(" ".join(f32text(v) for v in r) + "   # x y z t0 f0 fx fy fz")
    lines.append("<anchor_moment>")
    for r in moments:   # one record over two lines
        w = [f32text(v) if q < 5 or mech == "moment" else repr(float(v)) for q, v in enumerate(r)]
        lines += [" ".join(w[:4]), " ".join(w[4:])]
    write(os.path.join(tmp, "SeisSource.conf"), lines)
