"""The CPU restatement of the reference's LSQR (inv.LSQR/mod_LSQR.f90 slsqr, lgtsol)
pinned against an independent implementation of the same published algorithm (Paige and
Saunders 1982; scipy.sparse.linalg.lsqr): from x = 0 both produce the same iterates in
exact arithmetic.  In floating point the iterates of any two implementations (or of one
implementation on a row-permuted copy of the system) drift apart in the middle of the
iteration: without reorthogonalisation LSQR amplifies rounding there (on the systems below
scipy against itself on permuted rows differs by 2e-5 at iteration 16).  So the pin checks
what is well-conditioned: the first iterates (1e-10), the residual norm phibar = |b - A x|
at every iteration count (1e-7), and converged solutions (against the dense least-squares
solution, within the stopping tolerance).  The edge cases of the reference (zero
right-hand side: rho = 0 ends the iteration; repeated column indices in a row add) and the
standard errors of lgtsol are checked directly."""
import numpy as np
import pytest

sp = pytest.importorskip("scipy.sparse")
splinalg = pytest.importorskip("scipy.sparse.linalg")


def _system(m, n, density, seed):
    rng = np.random.default_rng(seed)
    A = sp.random(m, n, density=density, random_state=seed, format="csr")
    A.sort_indices()
    return A, rng.normal(size=m)


@pytest.mark.parametrize("k", [1, 3, 6, 12, 16, 40])
def test_iterates_match_paige_saunders(k, oracle_mod):
    A, b = _system(300, 120, 0.1, 1)
    r = oracle_mod.lsqr(A.indptr, A.indices, A.data, b, A.shape[1], atol=0.0, btol=0.0, maxit=k)
    s = splinalg.lsqr(A, b, atol=0.0, btol=0.0, conlim=0.0, iter_lim=k)
    assert r["itct"] == k == s[2]
    if k <= 6:
        np.testing.assert_allclose(r["x"], s[0], rtol=0, atol=1e-10 * np.abs(s[0]).max())
    # phibar is the residual norm |b - A x| of the iterate, in both implementations
    assert r["phibar"] == pytest.approx(np.linalg.norm(b - A @ r["x"]), rel=1e-7)
    assert r["phibar"] == pytest.approx(s[3], rel=1e-7)
    assert r["anorm"] == pytest.approx(np.sqrt((A.data ** 2).sum()), rel=1e-14)


def test_converged_solution_and_errors(oracle_mod):
    A, b = _system(400, 90, 0.08, 2)
    lam = 0.3  # damping rows as the inversion appends them (lamb on the diagonal, rhs 0)
    D = sp.identity(90, format="csr") * lam
    G = sp.vstack([A, D], format="csr")
    rhs = np.concatenate([b, np.zeros(90)])
    r = oracle_mod.lsqr(G.indptr, G.indices, G.data, rhs, 90)
    want = np.linalg.lstsq(G.toarray(), rhs, rcond=None)[0]
    assert r["flag"] == 1 and 1 < r["itct"] < 200
    assert r["test1"] <= 1e-7 or r["test2"] <= 1e-7
    np.testing.assert_allclose(r["x"], want, rtol=0, atol=1e-5 * np.abs(want).max())
    # lgtsol: sqrt(res2 / max(nrow - nvar, 1) * sig)
    np.testing.assert_allclose(r["serr"], np.sqrt(r["res2"] / (G.shape[0] - 90) * r["sig"]), rtol=1e-15)
    assert r["res2"] == r["phibar"]


def test_zero_rhs_and_repeated_columns(oracle_mod):
    A, _ = _system(50, 20, 0.2, 3)
    r = oracle_mod.lsqr(A.indptr, A.indices, A.data, np.zeros(50), 20)
    assert r["flag"] == 2 and r["itct"] == 0 and not np.any(r["x"])
    # a row whose column appears twice acts as the sum of the two entries
    rp = np.array([0, 2, 3, 5])
    ci = np.array([0, 0, 1, 1, 0])
    va = np.array([1.0, 2.0, 1.0, 0.5, 1.0])
    b = np.array([3.0, 1.0, 2.0])
    r = oracle_mod.lsqr(rp, ci, va, b, 2, atol=0, btol=0, maxit=2)
    dense = np.array([[3.0, 0.0], [0.0, 1.0], [1.0, 0.5]])
    np.testing.assert_allclose(r["x"], np.linalg.lstsq(dense, b, rcond=None)[0], rtol=1e-12)
