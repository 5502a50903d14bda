"""ORACLE — test infrastructure, never the product.

CPU restatement of the reference's kernel assembly onto inversion blocks
(code/srcF.kernel/SI_ker2assm.F90): the projection B(n) = sum over block n's pixels of
K(i,j,k) * volume(m,n) in single precision, pixel by pixel in the block file's order
(:306-323), the running sums S(n) += |B(n)| (:318-321), the C scaling and the compact rows
of export_G_compact (:545-571).  numpy float32 operations vectorised over the blocks keep
each block's sequential order, so the result is the reference's rounding.  Only the tests
use it.  Parity is pinned only by the source text: the reference ships no block files or
kernel rows.
"""
from __future__ import annotations

import struct

import numpy as np


def project(kernel, volume, num_of_pix, indx_of_pix):
    """kernel (ki, kj, kk); volume (max_pix, num_blk); num_of_pix (num_blk);
    indx_of_pix (3, max_pix, num_blk), 1-based.  Returns B (num_blk) float32."""
    K = np.asarray(kernel, np.float32)
    vol = np.asarray(volume, np.float32)
    npix = np.asarray(num_of_pix)
    pix = np.asarray(indx_of_pix) - 1
    max_pix, nblk = vol.shape
    B = np.zeros(nblk, np.float32)
    for m in range(max_pix):
        act = npix > m
        if not act.any():
            continue
        i, j, k = pix[0, m, act], pix[1, m, act], pix[2, m, act]
        B[act] = B[act] + K[i, j, k] * vol[m, act]
    return B


def compact(B, C, ker0):
    """B scaled by C in SP, then the 1-based indices and values with |B*C| > ker0."""
    Bs = np.asarray(B, np.float32) * np.float32(C)
    idx = np.nonzero(np.abs(Bs) > np.float32(ker0))[0]
    return idx + 1, Bs[idx]


def row_file_bytes(nblk, ker0, idx, val) -> bytes:
    """The bytes of one compact row file: Fortran unformatted records (4-byte markers) of
    (num_blk, ker0), (ncoef) and the (index, value) pairs."""
    def rec(b: bytes) -> bytes:
        return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))
    pairs = b"".join(struct.pack("<if", int(i), float(v)) for i, v in zip(idx, np.asarray(val, np.float32)))
    return rec(struct.pack("<if", int(nblk), float(np.float32(ker0)))) + rec(struct.pack("<i", len(idx))) + rec(pairs)


def sum_file_bytes(S) -> bytes:
    S = np.asarray(S, np.float32)
    def rec(b: bytes) -> bytes:
        return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))
    return rec(struct.pack("<i", S.size)) + rec(S.astype("<f4").tobytes())
