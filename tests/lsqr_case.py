"""A seeded synthetic inversion in the reference's input formats (kernel row files, data
list, smoothing operator, standard-input answers) for the inversion program's tests."""
import os

import numpy as np

from fwant_gb300 import inputs

NBLK, NCMP = 40, 2
SETTINGS = dict(num_cmp=NCMP, nsta=1, weig_sta=0.5, nevt=1, weig_evt=0.25, lamb=0.3, eta=0.8, ker_thres=1e-3,
                data_thres=5.0)


def make_case(root, loc=False, ndata=30, seed=4):
    rng = np.random.default_rng(seed)
    lines = ["# kernel files, datum, weight, station, event" + (", location id and weight" if loc else "")]
    for d in range(ndata):
        files = []
        for k in range(NCMP):
            n = int(rng.integers(3, 15))
            idx = rng.choice(np.arange(1, NBLK + 1), size=n, replace=False)
            coef = rng.normal(size=n).astype(np.float32)
            coef[rng.random(n) < 0.2] *= 1e-4  # some below the kernel threshold
            p = os.path.join(root, f"G{d:03d}_{k}.bin")
            inputs.write_kernel_row_file(p, NBLK, idx, coef, ker0=float(rng.random()))
            files.append(p)
        rhs = 9.0 if d == 7 else rng.normal()  # measurement 7 above the data threshold
        w = rng.uniform(0.5, 2.0)
        sta = int(rng.integers(1, 6)) * (1 if rng.random() < 0.8 else -1)
        evt = int(rng.integers(1, 5))
        row = files + [repr(float(np.float32(rhs))), repr(float(np.float32(w))), str(sta), str(evt)]
        if loc:
            row += [str(int(rng.integers(1, 4))), repr(float(rng.uniform(0.5, 1.5)))]
        lines.append(" ".join(row))
    lst = os.path.join(root, "data.lst")
    with open(lst, "w") as f:
        f.write("\n".join(lines) + "\n")
    sm = os.path.join(root, "smooth.txt")
    inputs.write_smoothing_file(sm, NBLK, [([i, i + 1], [-1.0, 1.0]) for i in range(1, NBLK)])
    s = SETTINGS
    if not loc:
        answers = [1, f"{s['lamb']} {s['eta']}", s["num_cmp"], f"{s['nsta']} {s['weig_sta']}",
                   f"{s['nevt']} {s['weig_evt']}", lst, sm, f"{s['ker_thres']} {s['data_thres']}"]
    else:
        answers = [1, lst, sm, s["num_cmp"], f"{s['nsta']} {s['weig_sta']}", f"{s['nevt']} {s['weig_evt']}", "1 0.7",
                   f"{s['lamb']} {s['eta']}", f"{s['ker_thres']} {s['data_thres']}"]
    return lst, sm, "\n".join(str(a) for a in answers) + "\n"


def oracle_system(lst, sm, loc=False):
    from oracle import inversion_oracle as io
    s = SETTINGS
    return io.assemble(lst, sm, s["num_cmp"], s["nsta"], s["weig_sta"], s["nevt"], s["weig_evt"], s["lamb"], s["eta"],
                       s["ker_thres"], s["data_thres"], nloc=1 if loc else 0, weig_loc=0.7 if loc else 0.0)
