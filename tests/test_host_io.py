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
