"""The medium preprocessor program end to end on the GPU: fwant_media reads SeisFD3D.conf,
the grid's coord file, the media configuration and a model file in each of the reference's
formats (ascii cart1d / interface / layered, NetCDF composite / volume / verpoly) and writes
media_mpi000000.nc; its lambda, mu and rho equal the restatement's evaluation of the arrays
the reference's readers would have formed from the same files (unit factors and the
degree-to-radian conversion applied in the readers' precision)."""
import os
import subprocess

import numpy as np
import pytest

import media_case as mc

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_media")
f32 = np.float32


def _deg(rad):
    return (np.asarray(rad, np.float64) * 180.0 / np.pi).astype(f32)


def _rad(deg):
    """the readers' conversion: real(SP) * PI / 180.0_DP, stored in SP"""
    return (np.asarray(deg, f32).astype(np.float64) * np.pi / 180.0).astype(f32)


def _scaled(a, f):
    return (np.asarray(a, f32).astype(np.float64) * f).astype(f32)


def _write_model(root, name, call, perturbed):
    """write one set-up call as the reference's file; returns (type, format, file) and the
    set-up call the readers' arrays give"""
    from fwant_gb300 import inputs
    meth, args = call
    path = os.path.join(root, name)
    if meth == "set_cart1d":
        d, vp, vs, rho = args
        km = [(np.asarray(a, np.float64) / 1000.0).astype(f32) for a in (d, rho, vp, vs)]
        inputs.write_cart1d_file(path, *km, meaning="depth", units=(1000.0, 1000.0, 1000.0))
        dd, rr, pp, ss = (_scaled(a, 1000.0) for a in km)
        return ("cart1d", "ascii", path), ("set_cart1d", (dd, pp, ss, rr))
    if meth == "set_layers":
        kind, x, y, z, h, vp, vs, rho = args[:8]
        xd, yd = _deg(x), _deg(y)
        if kind == mc.INTERFACE:
            inputs.write_layer_file(path, "interface", xd, yd, z, vp, vs, rho)
            hh = np.zeros_like(z)
            hh[:, :, :-1] = z[:, :, :-1] - z[:, :, 1:]
            return ("interface", "ascii", path), ("set_layers", (kind, _rad(xd), _rad(yd), z, hh, vp, vs, rho))
        if kind == mc.LAYERED:
            d = np.cumsum(h, axis=2, dtype=f32)
            inputs.write_layer_file(path, "layered", xd, yd, d, vp, vs, rho, meaning="depth")
            hd = np.empty_like(d)
            hd[:, :, 0] = d[:, :, 0]
            hd[:, :, 1:] = d[:, :, 1:] - d[:, :, :-1]
            return ("layered", "ascii", path), ("set_layers", (kind, _rad(xd), _rad(yd), None, hd, vp, vs, rho))
        inputs.write_composite_nc(path, xd, yd, h, vp, vs, rho, *args[8:])
        return ("composite", "nc", path), ("set_layers", (kind, _rad(xd), _rad(yd), None, h, vp, vs, rho, *args[8:]))
    if meth == "set_volume":
        p, x, y, rz, rz0, vp, vs, rho = args
        xd, yd = _deg(x), _deg(y)
        inputs.write_volume_nc(path, xd, yd, rz, rz0, vp, vs, rho)
        return ("volume", "nc", path), ("set_volume", (p, _rad(xd), _rad(yd), rz, rz0, vp, vs, rho))
    p, x, y, rz, rz0, *rest = args
    xd, yd = _deg(x), _deg(y)
    inputs.write_verpoly_nc(path, xd, yd, rz, rz0, *rest)
    return ("verpoly", "nc", path), ("set_verpoly", (p, _rad(xd), _rad(yd), rz, rz0, *rest))


def _write_grid(root, x, y, z):
    from scipy.io import netcdf_file
    with netcdf_file(os.path.join(root, "coord_mpi000000.nc"), "w", version=1) as f:
        for d, a in (("I", x), ("J", y), ("K", z)):
            f.createDimension(d, a.size)
        for v, d, a in (("x", "I", x), ("y", "J", y), ("z", "K", z)):
            f.createVariable(v, "f4", (d,))[:] = a


@pytest.mark.parametrize("kind,perturb", [(mc.CART1D, mc.VOLUME), (mc.INTERFACE, mc.VERPOLY), (mc.LAYERED, None),
                                          (mc.COMPOSITE, None), (mc.VOLUME, None), (mc.VERPOLY, mc.VOLUME)])
def test_program_matches_restatement(kind, perturb, tmp_path, oracle_mod, native_lib):
    from scipy.io import netcdf_file

    from fwant_gb300 import inputs
    from oracle import oracle as orc
    assert os.path.exists(EXE), "fwant_media not built"
    ni, nj, nk, half = 14, 12, 10, (1, 1, 1)
    root = str(tmp_path)
    x, y, z, zt = mc.grid(ni, nj, nk, seed=11)
    calls = mc.case(kind, x, y, z, zt, seed=12, perturb=perturb)
    bg, bg_call = _write_model(root, "background.mdl", calls[0], 0)
    pt, oracle_calls = None, [bg_call]
    if perturb is not None:
        pt, p_call = _write_model(root, "perturbed.mdl", calls[1], 1)
        oracle_calls.append(p_call)
    _write_grid(root, x, y, z)
    inputs.write_media_conf(os.path.join(root, "SeisMedia.conf"), bg, pt, half)
    with open(os.path.join(root, "SeisFD3D.conf"), "w") as f:
        f.write(f"ni = {ni}\nnj = {nj}\nnk = {nk}\nstept = 0.05\ndims = 1 1 1\nGRID_ROOT = {root}\n"
                f"MEDIA_CONF = {root}/SeisMedia.conf\nMEDIA_ROOT = {root}\n")
    r = subprocess.run([EXE], capture_output=True, text=True, cwd=root)
    assert r.returncode == 0, r.stderr
    assert "Maximum allowed time step is" in r.stdout
    o = mc.feed(orc.MediaOracle(ni, nj, nk, x, y, z, zt, half), oracle_calls)
    want = o.eval()
    dt = o.stept_check()
    exact = kind not in (mc.COMPOSITE, mc.VERPOLY) and perturb != mc.VERPOLY
    with netcdf_file(os.path.join(root, "media_mpi000000.nc"), "r", mmap=False) as f:
        assert list(f.variables) == ["rho", "lambda", "mu"]
        assert f.dimensions["I"] == ni + 6 and f.nk2 == nk + 3 and list(f.count) == [ni + 6, nj + 6, nk + 6]
        for name, w in (("lambda", want[0]), ("mu", want[1]), ("rho", want[2])):
            got = np.asarray(f.variables[name][:]).transpose(2, 1, 0)
            if exact:
                np.testing.assert_array_equal(got, w, err_msg=name)
            else:
                np.testing.assert_allclose(got, w, rtol=4e-6, atol=0, err_msg=name)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("located on")][0]
    assert tuple(int(v) for v in line.split()[2:5]) == dt[1]
    assert ("Serious Error" in r.stdout) == (dt[0] < 0.05)


def test_program_rejects_bad_models(tmp_path, native_lib):
    from fwant_gb300 import inputs
    root = str(tmp_path)
    x, y, z, zt = mc.grid(6, 6, 6)
    _write_grid(root, x, y, z)
    bad = os.path.join(root, "bad.mdl")
    # Vp**2 <= 2 Vs**2 fails layer1d_read's check
    inputs.write_cart1d_file(bad, [0.0, 100.0], [2.0, 2.0], [3.0, 3.0], [2.5, 2.5], units=(1000.0, 1000.0, 1000.0))
    inputs.write_media_conf(os.path.join(root, "m.conf"), ("cart1d", "ascii", bad))
    with open(os.path.join(root, "SeisFD3D.conf"), "w") as f:
        f.write(f"ni = 6\nnj = 6\nnk = 6\nstept = 0.05\nGRID_ROOT = {root}\nMEDIA_CONF = {root}/m.conf\n"
                f"MEDIA_ROOT = {root}\n")
    r = subprocess.run([EXE], capture_output=True, text=True, cwd=root)
    assert r.returncode != 0 and "Vp**2 < 2Vs**2" in r.stderr
    inputs.write_media_conf(os.path.join(root, "m.conf"), ("cart1d", "nc", bad))
    r = subprocess.run([EXE], capture_output=True, text=True, cwd=root)
    assert r.returncode != 0 and "only ascii input" in r.stderr
