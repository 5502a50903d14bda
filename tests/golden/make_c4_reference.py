"""Generate tests/golden/c4_fp64_reference.npz: the FP64 reference of the config-4
precision study (tests/c4_study.py) from the double-precision CPU restatement.

Both simulations of the station pair run in double with the metric kept in double; the
SGT frames of the kernel block are taken from the double fields (rounded to FP32, the
precision of sgt_ files), and the ZZ kernel is accumulated in FP64 by the restatement of
sgt2scatter3 + scatter2kernel.  Stored: the velocity seismograms of both simulations and
the four kernels (FP32 is ample for errors measured at 1e-7 and above).

About an hour on 8 cores.  Run from the repository root:
    python tests/golden/make_c4_reference.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import c4_study as S  # noqa: E402
from fwant_gb300 import inputs  # noqa: E402
from oracle import oracle as O  # noqa: E402

STRESS = ("Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz")


def simulate(m):
    o = O.Oracle(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface, dbl=True)
    inputs.attach(o, m, metric=O.metric(m.x, m.y, m.z, full=True))
    frames = np.zeros((6, S.KNT, S.NPTS), np.float32)
    sl = tuple(slice(S.SUBS[d] - 1, S.SUBS[d] - 1 + S.SUBT[d] * S.SUBC[d], S.SUBT[d]) for d in range(3))
    t0 = time.time()
    for step in range(1, S.NT + 1):
        o.run(1)
        if step % S.TINV == 0:
            f = step // S.TINV - 1
            for c, name in enumerate(STRESS):
                frames[c, f] = o.get_field(name)[sl].transpose(2, 1, 0).reshape(-1)
        if step % 100 == 0:
            print(f"{m.name}: step {step} ({time.time() - t0:.0f} s)", flush=True)
    seis = o.get_seismo()
    o.close()
    return seis, frames


def main():
    O.build()
    O.set_threads(os.cpu_count() or 1)
    ma, mb = S.models()
    seis_a, sgt_a = simulate(ma)
    seis_b, sgt_b = simulate(mb)
    lam, mu = S.block_media(ma)
    kdt, nt1, nt2 = S.window(ma.stept)
    series = O.sgt2scatter3(lam, mu, [None, None, sgt_b], sgt_a, kdt, mode=1)
    v, u = S.kernel_waveforms(seis_a[2, :, 1], ma.stept)
    ker = O.scatter2kernel(v, u, series[2], series[4], kdt, nt1, nt2, S.SGT_M0, mode=1)
    np.savez_compressed(os.path.join(HERE, "c4_fp64_reference.npz"),
                        seis_a=seis_a[:3].astype(np.float32), seis_b=seis_b[:3].astype(np.float32),
                        kernels=np.stack(ker).astype(np.float32), nt=S.NT, tinv=S.TINV)


if __name__ == "__main__":
    main()
