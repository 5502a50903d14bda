"""Splits a one-rank input set (coord_, metric_, media_, source_ and station_mpi000000.nc)
into the per-rank files the reference's preprocessors write for dims (da, db, dc)
(set_mpi_subfix, code/srcF/mod_mpi.F90:415-423), for the tests of `fwant_prep stitch`:

* grid files hold each rank's local arrays with ghosts, global points a*ni + l,
  l = 0 .. ni+5 (swmpi_globi, mod_mpi.F90:450-454); `poison` adds 1e6 to the ghost values
  a rank holds for a neighbour's interior, which the stitcher must never read;
* source files list every source whose centre lies in the rank's points with ghosts,
  with local indices (seis3d_source.F90:186-293);
* station files list the receivers of the rank's interior, indx local, gindx global
  (seis3d_station.F90:64-105)."""
import os

import numpy as np

LENFD = 3


def _read(path):
    from scipy.io import netcdf_file
    with netcdf_file(path, "r", mmap=False) as f:
        return ({k: (np.array(v[:]), v.dimensions, v.typecode()) for k, v in f.variables.items()},
                dict(f.dimensions), dict(f._attributes))


def split(src_root, dst_root, dims, n, poison=True):
    from scipy.io import netcdf_file
    os.makedirs(dst_root, exist_ok=True)
    da, db, dc = dims
    ranks = [(a, b, c) for a in range(da) for b in range(db) for c in range(dc)]
    axis = {"I": 0, "J": 1, "K": 2}

    def suffix(r):
        return "mpi%02d%02d%02d" % r

    for name in ("coord", "metric", "media"):
        vars_, dimlens, atts = _read(os.path.join(src_root, f"{name}_mpi000000.nc"))
        for r in ranks:
            with netcdf_file(os.path.join(dst_root, f"{name}_{suffix(r)}.nc"), "w", version=1) as f:
                for dn in ("I", "J", "K"):
                    f.createDimension(dn, n[axis[dn]] + 2 * LENFD)
                for k, v in atts.items():
                    setattr(f, k, v)
                for var, (a, vdims, tc) in vars_.items():
                    sl = tuple(slice(r[axis[d]] * n[axis[d]], r[axis[d]] * n[axis[d]] + n[axis[d]] + 2 * LENFD)
                               for d in vdims)
                    loc = np.array(a[sl], dtype=a.dtype)
                    if poison:
                        for q, d in enumerate(vdims):
                            ax = axis[d]
                            idx = [slice(None)] * loc.ndim
                            if r[ax] > 0:
                                idx[q] = slice(0, LENFD)
                                loc[tuple(idx)] += 1.0e6
                            if r[ax] < dims[ax] - 1:
                                idx[q] = slice(n[ax] + LENFD, n[ax] + 2 * LENFD)
                                loc[tuple(idx)] += 1.0e6
                    out = f.createVariable(var, tc, vdims)
                    out[:] = loc

    vars_, dimlens, atts = _read(os.path.join(src_root, "source_mpi000000.nc"))
    for r in ranks:
        off = np.array([r[q] * n[q] for q in range(3)])
        with netcdf_file(os.path.join(dst_root, f"source_{suffix(r)}.nc"), "w", version=1) as f:
            f.createDimension("geo_dimension", 3)
            for k, v in atts.items():
                setattr(f, k, v)
            for kind in ("force", "moment"):
                key = f"{kind}_indx"
                if key not in vars_:
                    setattr(f, f"number_of_{kind}", np.int32(0))
                    continue
                g = vars_[key][0]
                loc = g - off[None, :]
                keep = np.all((loc >= 1) & (loc <= np.array(n) + 2 * LENFD), axis=1)
                setattr(f, f"number_of_{kind}", np.int32(keep.sum()))
                if not keep.any():
                    continue
                f.createDimension(f"{kind}_point", int(keep.sum()))
                f.createDimension(f"{kind}_time_window", dimlens[f"{kind}_time_window"])
                for var, (a, vdims, tc) in vars_.items():
                    if not var.startswith(kind) and var not in ("Fx", "Fy", "Fz", "Mxx", "Myy", "Mzz", "Mxy",
                                                                   "Mxz", "Myz"):
                        continue
                    if vdims[0] == f"{kind}_point":
                        vals = (loc if var == key else a)[keep]
                    elif vdims[0] == f"{kind}_time_window" or vdims == ("force_time_window",):
                        vals = a
                    else:
                        continue
                    out = f.createVariable(var, tc, vdims)
                    out[:] = vals

    vars_, dimlens, atts = _read(os.path.join(src_root, "station_mpi000000.nc"))
    g = vars_["indx"][0]
    for r in ranks:
        off = np.array([r[q] * n[q] for q in range(3)])
        loc = g - off[None, :]
        keep = np.all((loc >= LENFD + 1) & (loc <= np.array(n) + LENFD), axis=1)
        with netcdf_file(os.path.join(dst_root, f"station_{suffix(r)}.nc"), "w", version=1) as f:
            f.createDimension("num_pt", None)
            f.createDimension("geo_dim", 3)
            f.createDimension("twoelem", 2)
            for k, v in atts.items():
                setattr(f, k, v)
            for var, (a, vdims, tc) in vars_.items():
                out = f.createVariable(var, tc, vdims)
                if keep.any():
                    out[:int(keep.sum())] = (loc if var == "indx" else a)[keep]
