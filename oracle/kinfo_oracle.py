"""CPU restatement of the reference's kernel statistics, SI_ker2info
(code/srcF.kernel/SI_ker2info.F90) — test infrastructure only: the oracle the GPU pass
(fwant_kerinfo, `fwant_ker --info`) is checked against.  Parity unpinned against reference
outputs (the reference's Fortran is not built here); the restatement is pinned by a
hand-worked case in tests/test_kinfo_oracle.py.

Per pick of an event (SI_ker2info.F90:271-289), with K the four kernel volumes
(phase_Vp, amplitude_Vp, phase_Vs, amplitude_Vs; slots ap, aq, bp, bq) in single precision:
    S_q = S_q + |K_q|                      never reset
    M_q = M_q + 1 where |K_q| > K0_q        reset at the start of each event with picks (:227)
At the end of such an event (:294-334), point by point:
    M_ap >= 1: N_ap += 1; record N_ap <- (KSTNM, KEVNM, M_ap) in the ap variables
    M_q >= 1 (q = aq, bp, bq): N_q += 1; record N_ap <- (KSTNM, KEVNM, M_q) in the q
        variables (the reference passes N_ap as the record index for all four); while
        N_ap = 0 that write is refused (record 0 does not exist) and nothing is stored
A name longer than its field (MAXKSTNM 8, MAXKEVNM 20, :33) or empty is not stored (the
library refuses the put, the reference ignores its status); the count M still is.
"""
import numpy as np

MAXKSTNM, MAXKEVNM = 8, 20


class KerInfo:
    """The statistics over volumes of `shape` (any layout; per point)."""

    def __init__(self, shape, thresholds):
        self.shape = tuple(shape)
        n = int(np.prod(self.shape))
        self.k0 = np.asarray(thresholds, np.float32).reshape(4)
        self.S = np.zeros((4, n), np.float32)
        self.N = np.zeros((4, n), np.int32)
        self.M = np.zeros((4, n), np.int32)
        self.rec_M, self.rec_sta, self.rec_evt = [], [], []   # per record: (4, n) / (4, n) object

    def add_pick(self, kernels):
        """kernels: the four volumes of one pick (SI_ker2info.F90:271-289)."""
        for q in range(4):
            a = np.abs(np.asarray(kernels[q], np.float32).reshape(-1))
            self.S[q] = self.S[q] + a                        # float32 + float32, rounded
            self.M[q] += (a > self.k0[q]).astype(np.int32)

    def end_event(self, station, event):
        """Close an event that had picks (SI_ker2info.F90:294-334), then reset M."""
        n = self.S.shape[1]
        sta = station if 0 < len(station) <= MAXKSTNM else None
        evt = event if 0 < len(event) <= MAXKEVNM else None
        hit = self.M >= 1
        self.N[0] += hit[0]
        nap = self.N[0]
        while len(self.rec_M) < int(nap.max(initial=0)):
            self.rec_M.append(np.zeros((4, n), np.int32))
            self.rec_sta.append(np.full((4, n), None, object))
            self.rec_evt.append(np.full((4, n), None, object))
        for q in range(4):
            if q > 0:
                self.N[q] += hit[q]
            pts = np.flatnonzero(hit[q] & (nap >= 1))
            for p in pts:
                r = nap[p] - 1
                self.rec_M[r][q, p] = self.M[q, p]
                if sta is not None:
                    self.rec_sta[r][q, p] = sta
                if evt is not None:
                    self.rec_evt[r][q, p] = evt
        self.M[:] = 0

    def records(self):
        return len(self.rec_M)

    def char_record(self, r, q, which):
        """The KSTNM (which 0) or KEVNM (which 1) characters of record r, slot q, as the file
        holds them: (points, width) bytes, the name then zeros."""
        width = MAXKSTNM if which == 0 else MAXKEVNM
        names = (self.rec_sta if which == 0 else self.rec_evt)[r][q]
        out = np.zeros((names.size, width), np.uint8)
        for p, s in enumerate(names):
            if s is not None:
                b = s.encode()
                out[p, :len(b)] = np.frombuffer(b, np.uint8)
        return out


def run(stations, thresholds, shape, read_kernels):
    """The whole program over parsed inputs: stations is a list of (KSTNM, events), an event
    (KEVNM, picks) with picks the list of pick directories in component order (empty: the
    event is skipped, :225); read_kernels(dir) returns the pick's four volumes."""
    info = KerInfo(shape, thresholds)
    for sta, events in stations:
        for evt, picks in events:
            if not picks:
                continue
            for d in picks:
                info.add_pick(read_kernels(d))
            info.end_event(sta, evt)
    return info
