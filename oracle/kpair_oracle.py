"""CPU restatement of SI_ker_pair (code/srcF.kernel/SI_ker_pair.F90), the kernels of one
source-receiver pair — test infrastructure only: the oracle that the GPU pair path
(fwant_sgtker_scatter_pair / _kernel_pair, `fwant_ker --pair`) is checked against.  Parity
unpinned against reference outputs (the Fortran is not built here); the filter is pinned
against scipy's direct-form filter with the same padding and history, the scatter against an
FP64 convolution (tests/test_kpair_oracle.py).

* stress2strain and sgt2scatter (:710-780): the single-precision program of
  oracle/sgtker_oracle.cpp (mode 0 of orc_sgt2scatter3: every value and accumulator FP32,
  operand order as the Fortran expressions) with the receiver SGT as its X component, whose
  series slots 0 and 3 are the pair's Sa and Sb;
* filter / filtfilt (:906-932): FP64 on the series between zero padding, NOD samples in
  front and 2 (NOD + 1) behind, each pass forcing y(1:NOD) = 0; results rounded to FP32
  where the reference assigns them to single-precision arrays (:840-904);
* scatter2kernel (:782-838): the single-precision program (mode 0 of orc_scatter2kernel).
"""
import numpy as np

from oracle import oracle as O


def scatter_pair(lam, mu, rsgt, ssgt, dt):
    """rsgt, ssgt: (6, knt, npts) stresses of the receiver and the source SGT.  Returns
    (Sa, Sb), (knt, npts) float64 holding FP32 values."""
    s = O.sgt2scatter3(lam, mu, [rsgt, None, None], ssgt, dt, mode=0)
    return s[0], s[3]


def pair_filter(series, b, a, mode):
    """filter (mode 1) / filtfilt (mode 2) of SI_ker_pair along axis 0 of (nt, ...), FP64."""
    b = np.asarray(b, np.float64)
    a = np.asarray(a, np.float64)
    x0 = np.asarray(series, np.float64)
    nt = x0.shape[0]
    nod = b.size - 1
    nel = nt + 3 * nod + 2
    rest = x0.shape[1:]

    def filt(x):
        y = np.zeros((nel + 1,) + rest)
        for n in range(nod + 1, nel + 1):
            yy = b[0] * x[n]
            for m in range(2, nod + 2):
                yy = (yy + b[m - 1] * x[n - m + 1]) - a[m - 1] * y[n - m + 1]
            y[n] = yy / a[0]
        return y

    x = np.zeros((nel + 1,) + rest)
    x[nod + 1: nod + 1 + nt] = x0
    y = filt(x)
    if mode == 2:
        w = np.zeros_like(y)
        w[1:] = y[nel:0:-1]
        z = filt(w)
        y = np.zeros_like(z)
        y[1:] = z[nel:0:-1]
    return y[nod + 1: nod + 1 + nt]


def kernel_pair(v, u, sa, sb, dt, nt1, nt2, sgt_m0, mode=0, b=None, a=None):
    """The four kernels (phase_Vp, amplitude_Vp, phase_Vs, amplitude_Vs) of the pair over
    frames nt1..nt2 (1-based) after the band's filter (mode 0 none, 1 one pass, 2
    forward-backward), float64 arrays holding FP32 values."""
    v = np.asarray(v, np.float32)
    u = np.asarray(u, np.float32)
    if mode:
        v = pair_filter(v, b, a, mode).astype(np.float32)
        u = pair_filter(u, b, a, mode).astype(np.float32)
        sa = pair_filter(sa, b, a, mode).astype(np.float32).astype(np.float64)
        sb = pair_filter(sb, b, a, mode).astype(np.float32).astype(np.float64)
    return O.scatter2kernel(v, u, sa, sb, dt, nt1, nt2, float(np.float32(sgt_m0)), mode=0)
