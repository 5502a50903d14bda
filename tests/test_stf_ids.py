"""Every source time function id the reference defines (src_stf / src_svf,
code/srcF/mod_src.F90:438-622): the values the solver tabulates per RK stage (host code
of the native library, no GPU) equal the oracle's FP32 restatement bit for bit, and both
refuse the same undefined (function, id) pairs, as the reference stops on them."""
import math

import numpy as np
import pytest

STF_IDS = (220, 200, 230, 100, 240, 250)       # src_stf cases
SVF_IDS = (120, 220, 200, 100, 230, 110, 240)  # src_svf cases
ALL_IDS = sorted(set(STF_IDS) | set(SVF_IDS) | {0, 999})


@pytest.mark.parametrize("stf_id", ALL_IDS)
@pytest.mark.parametrize("which", (0, 1))
def test_library_stf_equals_oracle(native_lib, oracle_mod, which, stf_id):
    import fwant_gb300 as fw
    defined = stf_id in (STF_IDS if which == 0 else SVF_IDS)
    stept = 0.0312
    # window start t0 / frequency or rise time f0 per family, and a time axis through
    # the whole window (negative times, the window edges, after the window)
    t0, f0 = {200: (1.0, 0.5), 220: (0.8, 0.3), 120: (0.8, 0.3)}.get(stf_id, (0.2, 0.9))
    n_bad = 0
    for n in range(0, 120):
        for frac in (0.0, 0.5, 1.0):
            t = (n + frac) * stept - 0.1
            ref = oracle_mod.stf(t, t0, f0, stf_id, n, stept) if which == 0 else \
                oracle_mod.svf(t, t0, f0, stf_id, n, stept)
            if not defined:
                assert math.isnan(ref)
                with pytest.raises(fw.FwantError):
                    fw.source_time_function(which, stf_id, t, t0, f0, n, stept)
                n_bad += 1
                continue
            got = fw.source_time_function(which, stf_id, t, t0, f0, n, stept)
            assert np.float32(got).tobytes() == np.float32(ref).tobytes(), (t, got, ref)
    assert (n_bad > 0) == (not defined)
