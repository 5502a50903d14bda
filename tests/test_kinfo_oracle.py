"""The kernel-statistics restatement (oracle/kinfo_oracle.py, SI_ker2info) pinned by a case
worked by hand from the reference's loops (code/srcF.kernel/SI_ker2info.F90:225-334):

two points, thresholds 1.0;
station STA1: event E1 with picks A and B, event E2 (a 25-character name) with pick C,
event E3 without picks; station LONGSTATION (11 characters): event E4 with pick D.

  A: Kap (2, 0.5)  Kaq (0.5, 3)  Kbp (0, 0)  Kbq (-2, -2)
  B: Kap (-1.5, 0) Kaq (1.0, 0)  Kbp (0, 0)  Kbq (0, 0)      |K| = K0 is not counted
  C: Kap (0, 5)    Kaq (4, 0)    Kbp (0, 0)  Kbq (0, 0)
  D: Kap (3, 3)    Kaq (0, 0)    Kbp (2, 0)  Kbq (0, 0)

E1: M_ap (2, 0), M_aq (0, 1), M_bq (1, 1).  Point 0: N_ap 1, record 1 ap = (2, STA1, E1);
N_bq 1, record 1 bq = (1, STA1, E1).  Point 1: N_ap stays 0, so N_aq and N_bq count 1 but
their record writes (index N_ap = 0) are refused.
E2: M_ap (0, 1), M_aq (1, 0).  Point 0: N_aq 1, record N_ap = 1 aq = (1, STA1, no event
name: too long).  Point 1: N_ap 1, record 1 ap = (1, STA1, no event name).
E4: M_ap (1, 1), M_bp (1, 0).  Point 0: N_ap 2, record 2 ap = (1, no station name, E4); N_bp 1,
record 2 bp = (1, -, E4).  Point 1: N_ap 2, record 2 ap = (1, -, E4).
"""
import numpy as np

from oracle import kinfo_oracle as KI

PICKS = {
    "A": [(2, 0.5), (0.5, 3), (0, 0), (-2, -2)],
    "B": [(-1.5, 0), (1.0, 0), (0, 0), (0, 0)],
    "C": [(0, 5), (4, 0), (0, 0), (0, 0)],
    "D": [(3, 3), (0, 0), (2, 0), (0, 0)],
}
STATIONS = [("STA1", [("E1", ["A", "B"]), ("EVENT_NAME_LONGER_THAN_20", ["C"]), ("E3", [])]),
            ("LONGSTATION", [("E4", ["D"])])]


def _run():
    read = lambda d: [np.array(v, np.float32) for v in PICKS[d]]  # noqa: E731
    return KI.run(STATIONS, [1.0] * 4, (2,), read)


def test_hand_worked_case():
    info = _run()
    np.testing.assert_array_equal(info.S, np.array([[6.5, 8.5], [5.5, 3.0], [2.0, 0.0], [2.0, 2.0]], np.float32))
    np.testing.assert_array_equal(info.N, [[2, 2], [1, 1], [1, 0], [1, 1]])
    assert info.records() == 2
    m1, m2 = info.rec_M
    np.testing.assert_array_equal(m1, [[2, 1], [1, 0], [0, 0], [1, 0]])
    np.testing.assert_array_equal(m2, [[1, 1], [0, 0], [1, 0], [0, 0]])
    s1, s2 = info.rec_sta
    e1, e2 = info.rec_evt
    assert list(s1[0]) == ["STA1", "STA1"] and list(e1[0]) == ["E1", None]
    assert list(s1[1]) == ["STA1", None] and list(e1[1]) == [None, None]
    assert list(s1[3]) == ["STA1", None] and list(e1[3]) == ["E1", None]
    assert list(s2[0]) == [None, None] and list(e2[0]) == ["E4", "E4"]
    assert list(s2[2]) == [None, None] and list(e2[2]) == ["E4", None]
    assert all(v is None for v in s2[1]) and all(v is None for v in s2[3])


def test_char_records_are_zero_padded():
    info = _run()
    c = info.char_record(0, 0, 0)
    assert c.shape == (2, 8)
    assert bytes(c[0]) == b"STA1\0\0\0\0" and bytes(c[1]) == b"STA1\0\0\0\0"
    e = info.char_record(0, 0, 1)
    assert e.shape == (2, 20) and bytes(e[0][:3]) == b"E1\0" and not e[1].any()


def test_sums_are_single_precision_in_pick_order():
    """S adds |K| in float32, pick after pick: 1e8 + 1 + 1 stays 1e8 in single precision."""
    info = KI.KerInfo((1,), [0.0] * 4)
    for v in (1.0e8, 1.0, 1.0):
        info.add_pick([np.array([v], np.float32)] * 4)
    info.end_event("S", "E")
    assert info.S[0, 0] == np.float32(1.0e8)
    assert info.N[0, 0] == 1 and info.rec_M[0][0, 0] == 3


def test_name_field_boundaries():
    """Names of exactly 8 (station) and 20 (event) characters are stored whole; one more
    character and the write is refused (the slot keeps its earlier name)."""
    info = KI.KerInfo((1,), [0.0] * 4)
    one = [np.array([1.0], np.float32)] * 4
    info.add_pick(one)
    info.end_event("ABCDEFGH", "E" * 20)
    assert bytes(info.char_record(0, 0, 0)[0]) == b"ABCDEFGH"
    assert bytes(info.char_record(0, 0, 1)[0]) == b"E" * 20
    info.add_pick(one)
    info.end_event("ABCDEFGHI", "F" * 21)           # record 2: names refused
    assert not info.char_record(1, 0, 0).any() and not info.char_record(1, 0, 1).any()
    assert info.rec_M[1][0, 0] == 1
