"""Host-side consumers of the assembled system, no GPU: the reference's text
formats reproduced byte for byte (golden files written by the reference
itself), the COO reader, and the check GMRES."""
import os

import numpy as np

from conftest import GOLDEN

TXT = os.path.join(GOLDEN, "text_unit3")


def _assembly():
    return np.load(os.path.join(GOLDEN, "assembly_unit3_p0_f0.npz"))


def test_text_formats_match_reference(fk, tmp_path):
    A = _assembly()
    assert fk.write_gb(tmp_path, A["rowptr"], A["col"], A["val"], A["B"], "coo") == 0
    assert open(tmp_path / "G.txt").read() == open(os.path.join(TXT, "G.txt")).read()
    assert fk.write_gb(tmp_path, A["rowptr"], A["col"], A["val"], A["B"], "csr") == 0
    for f in ("G_i.txt", "G_j.txt", "G_ij.txt", "B.txt"):
        assert open(tmp_path / f).read() == open(os.path.join(TXT, f)).read(), f


def test_positions_match_reference(fk, orc, tmp_path):
    m = np.load(os.path.join(GOLDEN, "mesh_unit3.npz"))
    order = np.argsort(m["node_int"][:, 0], kind="stable")
    gids = m["node_int"][order, 0]
    xy = m["node_dbl"][order, :2]
    b = orc.bvp(0)
    u = np.array([orc.coefficients(b, x, y)[0] for x, y in xy])
    assert fk.write_positions(tmp_path / "knot_position.txt", gids, xy, u) == 0
    assert open(tmp_path / "knot_position.txt").read() == open(os.path.join(TXT, "knot_position.txt")).read()


def test_read_coo_roundtrip(fk, tmp_path):
    A = _assembly()
    lines = open(os.path.join(TXT, "G.txt")).read()
    p = tmp_path / "G_in.txt"
    p.write_text(f"{len(A['col'])} {len(A['rowptr']) - 1}\n" + lines)
    rp, col, val = fk.read_gb_coo(p)
    assert np.array_equal(rp, A["rowptr"]) and np.array_equal(col, A["col"])
    assert np.allclose(val, A["val"], rtol=1e-7, atol=1e-30)


def test_gmres_solves_assembled_system(fk):
    A = _assembly()
    n = len(A["rowptr"]) - 1
    x, it, res, rc = fk.gmres(A["rowptr"], A["col"], A["val"], A["B"], tol=1e-11, max_iter=4000, restart=60)
    assert rc == 0 and res < 1e-10
    M = np.zeros((n, n))
    for i in range(n):
        M[i, A["col"][A["rowptr"][i]:A["rowptr"][i + 1]]] = A["val"][A["rowptr"][i]:A["rowptr"][i + 1]]
    assert np.allclose(M @ x, A["B"], atol=1e-8 * np.abs(A["B"]).max())


def _csr(M):
    rp, col, val = [0], [], []
    for i in range(M.shape[0]):
        nz = np.flatnonzero(M[i])
        col += nz.tolist()
        val += M[i, nz].tolist()
        rp.append(len(col))
    return np.array(rp, dtype=np.int32), np.array(col, dtype=np.int32), np.array(val)


def test_gmres_ilu0(fk):
    """fk_gmres_csr_pc with ILU(0): exact on a tridiagonal matrix (its LU has
    no fill-in), the Jacobi solution in fewer iterations on an assembled
    system, and the patterns it cannot use refused."""
    rng = np.random.default_rng(2)
    n = 200
    T = np.diag(4.0 + rng.uniform(0, 1, n)) + np.diag(rng.uniform(-1, 1, n - 1), 1) + \
        np.diag(rng.uniform(-1, 1, n - 1), -1)
    b = rng.standard_normal(n)
    x, it, res, rc = fk.gmres(*_csr(T), b, tol=1e-12, precond=fk.PC_ILU0)
    assert rc == 0 and it <= 2 and np.allclose(T @ x, b, atol=1e-10), (rc, it, res)
    A = _assembly()
    args = (A["rowptr"], A["col"], A["val"], A["B"])
    xj, itj, rj, rcj = fk.gmres(*args, tol=1e-11, max_iter=4000, restart=60, precond=fk.PC_JACOBI)
    xi, iti, ri, rci = fk.gmres(*args, tol=1e-11, max_iter=4000, restart=60, precond=fk.PC_ILU0)
    assert rcj == 0 and rci == 0 and ri < 1e-10
    assert np.allclose(xi, xj, atol=1e-8 * np.abs(xj).max())
    assert iti < itj, (iti, itj)
    # Jacobi through fk_gmres_csr_pc is fk_gmres_csr
    x0, it0, _, _ = fk.gmres(*args, tol=1e-11, max_iter=4000, restart=60)
    assert it0 == itj and np.array_equal(x0, xj)
    # a row without its diagonal, or columns out of order: FK_ERR_ARG
    rp, col, val = _csr(T)
    bad = col.copy()
    bad[rp[5]:rp[6]] = bad[rp[5]:rp[6]][::-1]
    assert fk.gmres(rp, bad, val, b, precond=fk.PC_ILU0)[3] == fk.FK_ERR_ARG
    T2 = T.copy()
    T2[7, 7] = 0.0
    assert fk.gmres(*_csr(T2), b, precond=fk.PC_ILU0)[3] == fk.FK_ERR_ARG
