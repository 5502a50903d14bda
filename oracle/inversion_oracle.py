"""ORACLE — test infrastructure, never the product.

Restatement of the inversion driver's system assembly and fit evaluation
(inv.LSQR/solver_damp_smooth.f90 :101-171 and result_evaluate :266-390; the location terms
of solver_damp_smo_loc.f90 :116-145, 380-389) in numpy, from the same inputs the program
reads.  The solve itself is `oracle.lsqr`."""
from __future__ import annotations

import struct

import numpy as np


def read_kernel_row_file(path):
    """(num_blk, ker0, idx, coef) of a Fortran unformatted kernel row file."""
    recs = []
    with open(path, "rb") as f:
        data = f.read()
    p = 0
    while p < len(data):
        n = struct.unpack_from("<i", data, p)[0]
        recs.append(data[p + 4:p + 4 + n])
        p += 8 + n
    nblk, ker0 = struct.unpack("<if", recs[0][:8])
    ncoef = struct.unpack("<i", recs[1][:4])[0]
    pairs = np.frombuffer(recs[2][:8 * ncoef], dtype=[("i", "<i4"), ("c", "<f4")])
    return nblk, ker0, pairs["i"].astype(np.int64), pairs["c"].copy()


def _records(list_path):
    out = []
    for raw in open(list_path).read().splitlines():
        t = raw[:300].strip()
        if t and not t.startswith("#"):
            out.append(t.split())
    return out


def assemble(list_path, smooth_path, num_cmp, nsta, weig_sta, nevt, weig_evt, lamb, eta, ker_thres, data_thres,
             nloc=0, weig_loc=0.0):
    """Rows of the system in the program's order: dict(rp, col (0-based), val, rhs, ncol,
    num_mval, num_sta, num_evt, num_loc, data_rows)."""
    recs = _records(list_path)
    nblk, max_st, max_ev, max_lo = 0, 0, 0, 0
    for w in recs:
        for k in range(num_cmp):
            nblk = read_kernel_row_file(w[k])[0]
        p = num_cmp + 2
        for k in range(nsta):
            max_st = max(max_st, abs(int(w[p + k])))
        p += nsta
        for k in range(nevt):
            max_ev = max(max_ev, abs(int(w[p + k])))
        p += nevt
        for k in range(nloc):
            max_lo = max(max_lo, abs(int(w[p + 2 * k])))
    num_mval = nblk * num_cmp
    ncol = num_mval + max_st + max_ev + max_lo
    rows, rhs = [], []
    for w in recs:
        cols, vals = _datum_row(w, num_cmp, nsta, weig_sta, nevt, weig_evt, nloc, weig_loc, ker_thres, num_mval,
                                max_st, max_ev)
        rhs32, wgt32 = np.float32(float(w[num_cmp])), np.float32(float(w[num_cmp + 1]))
        if abs(rhs32) > data_thres:
            continue
        vals = [v * np.float64(wgt32) for v in vals]
        if cols:
            rows.append((cols, vals))
            rhs.append(np.float64(np.float32(rhs32 * wgt32)))
    data_rows = len(rows)
    for i in range(ncol):
        rows.append(([i], [np.float64(lamb)]))
        rhs.append(0.0)
    tok = [l.split() for l in open(smooth_path).read().splitlines() if l.strip()]
    sm_nblk, nrow_sm = int(tok[0][0]), int(tok[0][1])
    for r in range(nrow_sm):
        w = tok[1 + r]
        nc = int(w[0])
        idx = [int(v) for v in w[1:1 + nc]]
        cf = [np.float32(float(v)) for v in w[1 + nc:1 + 2 * nc]]
        for k in range(num_cmp):
            rows.append(([i + k * sm_nblk - 1 for i in idx], [np.float64(c) * np.float64(eta) for c in cf]))
            rhs.append(0.0)
    rp = np.zeros(len(rows) + 1, np.int64)
    rp[1:] = np.cumsum([len(c) for c, _ in rows])
    col = np.array([c for cs, _ in rows for c in cs], np.int32)
    val = np.array([v for _, vs in rows for v in vs], np.float64)
    return dict(rp=rp, col=col, val=val, rhs=np.array(rhs, np.float64), ncol=ncol, num_mval=num_mval,
                num_sta=max_st, num_evt=max_ev, num_loc=max_lo, data_rows=data_rows, nblk=nblk, sm_nblk=sm_nblk)


def _datum_row(w, num_cmp, nsta, weig_sta, nevt, weig_evt, nloc, weig_loc, ker_thres, num_mval, num_sta, num_evt):
    cols, vals = [], []
    for k in range(num_cmp):
        nb, _, idx, coef = read_kernel_row_file(w[k])
        for i, c in zip(idx, coef):
            t = np.float64(c)
            if abs(t) > ker_thres:
                cols.append(int(i) + nb * k - 1)
                vals.append(t)
    p = num_cmp + 2
    for k in range(nsta):
        s = int(w[p + k])
        cols.append(num_mval + abs(s) - 1)
        vals.append(np.float64(abs(weig_sta) if s >= 0 else -abs(weig_sta)))
    p += nsta
    for k in range(nevt):
        e = int(w[p + k])
        cols.append(num_mval + num_sta + abs(e) - 1)
        vals.append(np.float64(abs(weig_evt) if e >= 0 else -abs(weig_evt)))
    p += nevt
    for k in range(nloc):
        cols.append(num_mval + num_sta + num_evt + int(w[p + 2 * k]) - 1)
        vals.append(np.float64(float(w[p + 2 * k + 1])) * np.float64(weig_loc))
    return cols, vals


def evaluate(list_path, smooth_path, sysd, mval, errx, num_cmp, nsta, weig_sta, nevt, weig_evt, data_thres,
             ker_thres, nloc=0, weig_loc=0.0):
    """result_evaluate: the statistics written to try.sum, as a dict."""
    fit = dvar = fit_w = dvar_w = 0.0
    nd = 0
    for w in _records(list_path):
        rhs32, wgt32 = np.float32(float(w[num_cmp])), np.float32(float(w[num_cmp + 1]))
        if abs(rhs32) > data_thres:
            continue
        nd += 1
        rw = np.float32(rhs32 * wgt32)
        dvar += float(rhs32) ** 2
        dvar_w += float(rw) ** 2
        cols, vals = _datum_row(w, num_cmp, nsta, weig_sta, nevt, weig_evt, nloc, weig_loc, ker_thres,
                                sysd["num_mval"], sysd["num_sta"], sysd["num_evt"])
        tmp = float(np.dot(vals, mval[cols])) if cols else 0.0
        fit += (tmp - float(rhs32)) ** 2
        fit_w += (tmp * float(wgt32) - float(rw)) ** 2
    nm = sysd["num_mval"]
    tok = [l.split() for l in open(smooth_path).read().splitlines() if l.strip()]
    smo = 0.0
    for r in range(int(tok[0][1])):
        w = tok[1 + r]
        nc = int(w[0])
        idx = np.array([int(v) for v in w[1:1 + nc]])
        cf = np.array([np.float32(float(v)) for v in w[1 + nc:1 + 2 * nc]], np.float64)
        for k in range(num_cmp):
            smo += float(np.dot(cf, mval[idx + k * sysd["sm_nblk"] - 1])) ** 2
    m = mval[:nm]
    st = mval[nm:nm + sysd["num_sta"]] * weig_sta
    ev = mval[nm + sysd["num_sta"]:nm + sysd["num_sta"] + sysd["num_evt"]] * weig_evt
    return {"percent of data_var reduction": (1 - fit / dvar) * 100,
            "percent of data_var reduction w weight": (1 - fit_w / dvar_w) * 100,
            "kai^2": fit_w, "kai^2/N": fit_w / nd, "number of data": nd,
            "error_variance (model_var?)": np.sqrt(np.sum(errx[:nm] ** 2) / nm),
            "smooth_norm": np.sqrt(smo / nm), "model_norm (model_var?)": np.sqrt(np.sum(m ** 2) / nm),
            "model_mean": m.mean(), "model_min": m.min(), "model_max": m.max(),
            "station_term_min": st.min() if st.size else 1e7, "station_term_max": st.max() if st.size else -1e7,
            "event_term_min": ev.min() if ev.size else 1e7, "event_term_max": ev.max() if ev.size else -1e7}
