"""The inversion program's inputs without a GPU: the system it assembles from the data
list, kernel row files (Fortran unformatted) and smoothing operator equals the restatement
of solver_damp_smooth's assembly bit for bit (both standard-input layouts, with and
without location terms); input errors are reported before any device call."""
import os
import subprocess

import numpy as np
import pytest

from lsqr_case import make_case, oracle_system

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "fwant_gb300", "bin", "fwant_lsqr")


@pytest.fixture(scope="module")
def exe(native_lib):
    assert os.path.exists(EXE), "fwant_lsqr not built"
    return EXE


@pytest.mark.parametrize("loc", [False, True])
def test_assembled_system_equals_restatement(loc, exe, tmp_path):
    lst, sm, answers = make_case(str(tmp_path), loc=loc)
    prefix = os.path.join(tmp_path, "sys")
    args = [exe, "--dump-system", prefix] + (["--loc"] if loc else [])
    r = subprocess.run(args, input=answers, capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert "omit large rhs" in r.stdout
    want = oracle_system(lst, sm, loc)
    rp = np.fromfile(prefix + ".rp", np.int64)
    np.testing.assert_array_equal(rp, want["rp"])
    np.testing.assert_array_equal(np.fromfile(prefix + ".col", np.int32), want["col"])
    np.testing.assert_array_equal(np.fromfile(prefix + ".val", np.float64), want["val"])
    np.testing.assert_array_equal(np.fromfile(prefix + ".rhs", np.float64), want["rhs"])
    assert want["data_rows"] == 29  # one of 30 measurements above the data threshold


def test_input_errors(exe, tmp_path):
    lst, sm, answers = make_case(str(tmp_path))

    def run(a):
        return subprocess.run([exe, "--dump-system", os.path.join(tmp_path, "x")], input=a, capture_output=True,
                              text=True, cwd=str(tmp_path))
    r = run("2\n" + answers.split("\n", 1)[1])
    assert r.returncode == 1 and "only Simple damping" in r.stderr
    r = run(answers.replace(lst, lst + ".missing"))
    assert r.returncode == 1 and "fnm_list open err" in r.stderr
    os.remove(os.path.join(tmp_path, "G003_1.bin"))
    r = run(answers)
    assert r.returncode == 1 and "open kernel err" in r.stderr
    r = run("\n".join(answers.splitlines()[:4]) + "\n")
    assert r.returncode == 1 and "ended early" in r.stderr
