"""Seeded inversion blocks over a kernel volume for the kernel-assembly tests: a partition
into bricks (ragged at the edges), each brick's pixels in a shuffled order, random cell
volumes, and one empty block."""
import numpy as np


def blocks(shape, brick=(4, 4, 4), seed=0):
    rng = np.random.default_rng(seed)
    ki, kj, kk = shape
    lists = []
    for k0 in range(0, kk, brick[2]):
        for j0 in range(0, kj, brick[1]):
            for i0 in range(0, ki, brick[0]):
                pts = [(i + 1, j + 1, k + 1) for k in range(k0, min(k0 + brick[2], kk))
                       for j in range(j0, min(j0 + brick[1], kj)) for i in range(i0, min(i0 + brick[0], ki))]
                rng.shuffle(pts)
                lists.append(pts)
    lists.insert(len(lists) // 2, [])   # an empty block
    nblk = len(lists)
    max_pix = max(len(p) for p in lists)
    volume = np.zeros((max_pix, nblk), np.float32)
    npix = np.zeros(nblk, np.int32)
    pixs = np.zeros((3, max_pix, nblk), np.int32)
    for n, pts in enumerate(lists):
        npix[n] = len(pts)
        for m, p in enumerate(pts):
            pixs[:, m, n] = p
            volume[m, n] = np.float32(rng.uniform(0.5, 2.0) * 1.0e6)
    return volume, npix, pixs


def kernels(shape, n, seed=1):
    rng = np.random.default_rng(seed)
    return [(rng.standard_normal(shape) * 10.0 ** rng.uniform(-12, -9, shape)).astype(np.float32) for _ in range(n)]
