"""Kernel assembly without a GPU: the restatement of SI_ker2assm's projection against a
plain loop and a known answer, the compact row format against the inversion's reader-side
writer, and the block-file checks of fwant_assm_create (made before any device work)."""
import numpy as np
import pytest

import assm_case as ac


def test_restatement_against_a_plain_loop():
    from oracle import assm_oracle as A
    shape = (7, 6, 5)
    volume, npix, pixs = ac.blocks(shape, brick=(3, 4, 2), seed=3)
    K = ac.kernels(shape, 1, seed=4)[0]
    want = np.zeros(volume.shape[1], np.float32)
    for n in range(volume.shape[1]):
        b = np.float32(0.0)
        for m in range(int(npix[n])):
            i, j, k = pixs[:, m, n] - 1
            b = np.float32(b + np.float32(K[i, j, k] * volume[m, n]))
        want[n] = b
    np.testing.assert_array_equal(A.project(K, volume, npix, pixs), want)
    # known answer: unit kernel and unit volumes give the pixel counts
    ones = np.ones_like(volume)
    np.testing.assert_array_equal(A.project(np.ones(shape, np.float32), ones, npix, pixs), npix.astype(np.float32))


def test_row_format_is_the_inversion_input(tmp_path):
    from oracle import assm_oracle as A

    from fwant_gb300 import inputs
    B = np.float32([0.5, -2.0, 1e-3, 3.0, -0.01])
    idx, val = A.compact(B, 2.0, 0.01)
    assert list(idx) == [1, 2, 4, 5] and val[1] == -4.0
    p = tmp_path / "row.unformat"
    inputs.write_kernel_row_file(str(p), 5, idx, val, ker0=0.01)
    assert p.read_bytes() == A.row_file_bytes(5, 0.01, idx, val)
    # no coefficient above the threshold: an empty third record
    p2 = tmp_path / "empty.unformat"
    inputs.write_kernel_row_file(str(p2), 5, [], [], ker0=100.0)
    assert p2.read_bytes() == A.row_file_bytes(5, 100.0, [], [])


def test_create_checks_the_block_file(native_lib):
    import fwant_gb300 as fw
    shape = (6, 5, 4)
    volume, npix, pixs = ac.blocks(shape, brick=(3, 3, 2))
    bad = pixs.copy()
    bad[2, 0, 1] = shape[2] + 1      # a pixel below the kernel volume
    with pytest.raises(fw.FwantError, match="outside the kernel volume"):
        fw.Assm(shape, volume, npix, bad)
    over = npix.copy()
    over[0] = volume.shape[0] + 1    # more pixels than max_pix
    with pytest.raises(fw.FwantError, match="outside 0..max_pix"):
        fw.Assm(shape, volume, over, pixs)
