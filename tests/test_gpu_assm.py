"""Kernel assembly onto inversion blocks on the GPU (SI_ker2assm's projection) against the
restatement in oracle/assm_oracle.py bit for bit: block values of 1-4 kernel volumes per
pick, the running sums of |B| over picks, kernels from host or device memory; and the
fwant_assm program end to end (kernel files, block file and list files in; compact rows,
sums and band widths out, byte for byte)."""
import os
import subprocess

import numpy as np
import pytest

import assm_case as ac

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_assm")
SHAPE = (24, 20, 16)


@pytest.mark.parametrize("nq", [1, 2, 4])
def test_projection_matches_restatement(nq, native_lib):
    import fwant_gb300 as fw
    from oracle import assm_oracle as A
    volume, npix, pixs = ac.blocks(SHAPE, seed=nq)
    a = fw.Assm(SHAPE, volume, npix, pixs)
    S = np.zeros((4, volume.shape[1]), np.float32)
    for pick in range(3):
        ks = ac.kernels(SHAPE, nq, seed=10 * pick + nq)
        got = a.project(ks)
        for q in range(nq):
            want = A.project(ks[q], volume, npix, pixs)
            np.testing.assert_array_equal(got[q], want)
            S[q] = S[q] + np.abs(want)
        assert a.last_ms() > 0
    np.testing.assert_array_equal(a.sums(), S)
    assert got[0][npix == 0].tolist() == [0.0]   # the empty block


def test_device_kernels_equal_host_kernels(native_lib):
    torch = pytest.importorskip("torch")
    import fwant_gb300 as fw
    volume, npix, pixs = ac.blocks(SHAPE, brick=(5, 3, 4), seed=7)
    ks = ac.kernels(SHAPE, 2, seed=8)
    host = fw.Assm(SHAPE, volume, npix, pixs).project(ks)
    dev = [torch.from_numpy(np.ascontiguousarray(k.reshape(-1, order="F"))).cuda() for k in ks]
    got = fw.Assm(SHAPE, volume, npix, pixs).project_device([t.data_ptr() for t in dev])
    np.testing.assert_array_equal(got, host)


def test_projection_errors(native_lib):
    import fwant_gb300 as fw
    volume, npix, pixs = ac.blocks(SHAPE)
    a = fw.Assm(SHAPE, volume, npix, pixs)
    ks = ac.kernels(SHAPE, 5)
    with pytest.raises(fw.FwantError):
        a.project(ks)                                   # at most 4 volumes
    with pytest.raises(fw.FwantError, match="device memory"):
        a.project_device([ks[0].ctypes.data])           # a host address is refused, not read


def test_device_volume_past_the_end_of_its_allocation_is_refused(native_lib):
    """A device pointer whose allocation ends before ki*kj*kk floats is refused on the host
    (cuMemGetAddressRange), before any launch could read past the allocation."""
    import ctypes as C
    import fwant_gb300 as fw
    volume, npix, pixs = ac.blocks(SHAPE)
    a = fw.Assm(SHAPE, volume, npix, pixs)
    nvol = SHAPE[0] * SHAPE[1] * SHAPE[2]
    rt = C.CDLL("libcudart.so.13")
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaMemset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
    rt.cudaFree.argtypes = [C.c_void_p]
    size = 8 << 20                      # a multiple of the allocation granularity
    base = C.c_void_p()
    assert rt.cudaMalloc(C.byref(base), size) == 0
    try:
        assert rt.cudaMemset(base, 0, size) == 0
        short = base.value + size - 4 * (nvol // 2)   # half a volume left in the allocation
        with pytest.raises(fw.FwantError, match="floats past the pointer"):
            a.project_device([short])
        got = a.project_device([base.value])         # the whole volume fits
        assert not np.any(got)
    finally:
        rt.cudaFree(base)


def _write_kernel(path, names, vols):
    from scipy.io import netcdf_file
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with netcdf_file(path, "w", version=1) as f:
        f.createDimension("I", SHAPE[0])
        f.createDimension("J", SHAPE[1])
        f.createDimension("K", SHAPE[2])
        for nm, v in zip(names, vols):
            x = f.createVariable(nm, "f4", ("K", "J", "I"))
            x[:] = np.asarray(v, np.float32).transpose(2, 1, 0)


def _f(v):
    return repr(float(np.float32(v)))


@pytest.mark.parametrize("kamu", [False, True, "lamu"], ids=["vpvs", "kamu", "lamu"])
def test_program_writes_the_reference_files(kamu, native_lib, tmp_path):
    from scipy.io import netcdf_file

    from oracle import assm_oracle as A
    tmp = str(tmp_path)
    volume, npix, pixs = ac.blocks(SHAPE, seed=11)
    nblk, max_pix = volume.shape[1], volume.shape[0]
    with netcdf_file(os.path.join(tmp, "blocks.nc"), "w", version=1) as f:
        f.createDimension("block", nblk)
        f.createDimension("max_pix", max_pix)
        f.createDimension("geo", 3)
        f.createVariable("volume", "f4", ("block", "max_pix"))[:] = volume.T
        f.createVariable("num_of_pix", "i4", ("block",))[:] = npix
        f.createVariable("indx_of_pix", "i4", ("block", "max_pix", "geo"))[:] = pixs.transpose(2, 1, 0)
    with open(os.path.join(tmp, "main.conf"), "w") as f:
        f.write("ni = 30\nnj = 26\nnk = 20\nnt = 10\nstept = 0.01\ndims = 1 1 1\nnumber_of_snap = 1\n"
                "snap_001 = 2 3 1 24 20 16 1 1 1 4 10 TV   # the kernel volume\n")
    with open(os.path.join(tmp, "TomoKernel.conf"), "w") as f:
        f.write(f"MAIN_CONF = {tmp}/main.conf\nsnap_id = 1\n")
    rot = "1 0 0 0 1 0 0 0 1"
    picks = ["ker/STA1/EV1/p1", "ker/STA1/EV1/p2", "./ker/STA2/EV3/p1"]
    with open(os.path.join(tmp, "evt1.lst"), "w") as f:
        f.write(f"EV1 1 0 1 0 0 0 {rot}\nsyn_x\nsyn_y\nsyn_z\n1 P2 10.0 20.0 {picks[0]}\n# a comment line\n"
                f"1 N 5.0 9.0 {picks[1]}\nEV2 0 0 0 0 0 0 {rot}\nsx\nsy\nsz\n")
    with open(os.path.join(tmp, "evt2.lst"), "w") as f:
        f.write(f"# events of STA2\nEV3 0 0 0 1 -1 0 {rot}\nsx\nsy\nsz\n2 P1 1.0 4.0 {picks[2]}\n")
    with open(os.path.join(tmp, "sta.lst"), "w") as f:
        f.write("STA1 evt1.lst\n# STA9 skipped.lst\nSTA2 evt2.lst\n")
    os.makedirs(os.path.join(tmp, "spool"))
    names = (["phase_la", "phase_mu"] if kamu == "lamu" else ["phase_ka", "phase_mu"]) if kamu else ["phase_Vp", "phase_Vs"]
    prefix = ("kernel_lamu_" if kamu == "lamu" else "kernel_kamu_") if kamu else "kernel_"
    ker = []
    for p, d in enumerate(picks):
        ks = ac.kernels(SHAPE, 2, seed=20 + p)
        ker.append(ks)
        _write_kernel(os.path.join(tmp, d, f"{prefix}001_mpi000000_n00000.nc"), names + ["amplitude_x"],
                      ks + [np.zeros(SHAPE, np.float32)])
    Ca, Cb = np.float32(2.0), np.float32(0.5)
    B0 = A.project(ker[0][0], volume, npix, pixs)
    ka = np.float32(np.median(np.abs(B0 * Ca)))    # about half the blocks above the threshold
    kb = np.float32(np.median(np.abs(A.project(ker[0][1], volume, npix, pixs) * Cb)))
    answers = f"sta.lst\nblocks.nc\nspool\n{_f(Ca)}, 1.0 {_f(Cb)}\n1.0\n{_f(ka)} 0.0 {_f(kb)} 0.0\n"
    args = [EXE, os.path.join(tmp, "TomoKernel.conf")] + ((["--lamu"] if kamu == "lamu" else ["--kamu"]) if kamu else [])
    r = subprocess.run(args, input=answers, capture_output=True, text=True, cwd=tmp)
    assert r.returncode == 0, r.stdout + r.stderr
    S = np.zeros((2, nblk), np.float32)
    band = [0, 0]
    for p, d in enumerate(picks):
        part = d.lstrip("./").replace("/", "_")
        for q, (C, k0, tag) in enumerate(((Ca, ka, "Kap"), (Cb, kb, "Kbp"))):
            B = A.project(ker[p][q], volume, npix, pixs)
            S[q] = S[q] + np.abs(B)
            idx, val = A.compact(B, C, k0)
            band[q] = max(band[q], len(idx))
            with open(os.path.join(tmp, "spool", f"{part}.{tag}.unformat"), "rb") as f:
                assert f.read() == A.row_file_bytes(nblk, k0, idx, val), (d, tag)
    for q, (C, tag) in enumerate(((Ca, "Kap"), (Cb, "Kbp"))):
        with open(os.path.join(tmp, "spool", f"inv_G_sum.{tag}.unformat"), "rb") as f:
            assert f.read() == A.sum_file_bytes(S[q] * C)
    conf = open(os.path.join(tmp, "spool", "inv_G_band.conf")).read().split("\n")
    got = {ln.split("=")[0].strip(): int(ln.split("=")[1]) for ln in conf if "=" in ln}
    assert got == {"max_band_width_Kap": band[0], "max_band_width_Kaq": 0, "max_band_width_Kbp": band[1],
                   "max_band_width_Kbq": 0}
    assert 0 < band[0] < nblk
