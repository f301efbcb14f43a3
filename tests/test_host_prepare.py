"""The product's host preprocessing (include/sbte.h) against the oracle.

Quadrature and geometry are computed by this package's own C++ code
(staticbtesolver_gb300/host/prepare.cpp, hash-map face matching); the oracle
restates the reference's loops.  Neighbour codes must agree exactly (they are
integers), geometry and quadrature to rounding.
"""
import numpy as np
import pytest

from conftest import SYNTH_CASES, TESTSH_CASES


@pytest.mark.parametrize("name", TESTSH_CASES + ["2Dcase2", "2Dcase5"] + SYNTH_CASES)
def test_preprocessing_matches_oracle(sbte, oracle_mod, get_case, name):
    c = get_case(name)
    p = sbte.Problem(*c.args())
    o = oracle_mod.Oracle(*c.args())
    assert (p.n_cell, p.n_dir, p.n_band, p.n_face, p.n_bc, p.dim) == (o.n_cell, o.n_dir, o.n_band, o.n_face,
                                                                      o.n_bc, o.dim)
    gq, oq = p.quadrature(), o.quadrature()
    np.testing.assert_allclose(gq["omega"], oq["omega"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(gq["s"], oq["s"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(gq["S"], oq["S"], rtol=1e-13, atol=1e-15)
    assert gq["solid_angle"] == oq["solid_angle"]
    assert gq["T_ref"] == oq["T_ref"]
    gg, og = p.geometry(), o.geometry()
    np.testing.assert_array_equal(gg["nbr"], og["nbr"])
    np.testing.assert_allclose(gg["volume"], og["volume"], rtol=1e-12)
    np.testing.assert_allclose(gg["area"], og["area"], rtol=1e-12)
    np.testing.assert_allclose(gg["normal"], og["normal"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(gg["centroid"], og["centroid"], rtol=1e-12, atol=1e-30)


def test_zero_sentinel_quirk(sbte, oracle_mod, tmp_path):
    """A boundary face without a boundary element keeps neighbour code 0 (a link to cell 0),
    as src/StaticBTESolver.cpp:631 does; both implementations must agree."""
    mesh = tmp_path / "m.mphtxt"
    # two triangles sharing an edge; only the left edge is listed as a boundary segment
    from staticbtesolver_gb300 import synth
    m = dict(dim=2, points=np.array([[0, 0], [1, 0], [1, 1], [0, 1.0]]), tri=np.array([[0, 1, 2], [0, 2, 3]]),
             seg=np.array([[0, 3]]), seg_ent=np.array([0]))
    synth.write_mphtxt(str(mesh), m)
    band = tmp_path / "b.dat"
    band.write_text("2677 39.9E-12 1.627E6 1\n")
    bc = tmp_path / "bc.dat"
    bc.write_text("1 #n\n\n#h\n0 1 301\n")
    args = (str(mesh), str(bc), str(band), 2, 8, 8, 300.0, 1e-8, 1e-8, 0.0)
    p, o = sbte.Problem(*args), oracle_mod.Oracle(*args)
    np.testing.assert_array_equal(p.geometry()["nbr"], o.geometry()["nbr"])
    assert (p.geometry()["nbr"] == 0).sum() >= 2


def test_bad_inputs_raise(sbte, tmp_path):
    with pytest.raises(sbte.BteError):
        sbte.Problem(str(tmp_path / "missing.mphtxt"), "x", "y", 2, 8, 8)
    band = tmp_path / "b.dat"
    band.write_text("2677 39.9E-12 1.627E6 1\n")
    bc = tmp_path / "bc.dat"
    bc.write_text("2 #n\n\n#h\n0 1 301\n1 1 299\n")
    with pytest.raises(sbte.BteError):
        sbte.Problem("100", str(bc), str(band), 4, 8, 1, 300, 1e-8)  # DM must be 2 or 3


def test_tempcell_writer_format(sbte, tmp_path):
    """The reference's field dump (src/StaticBTESolver.cpp:818-831): x/L_x y/L_y [z/L_z] T."""
    cen = np.array([[0.5e-8, 0.25e-8, 0.0], [1e-8, 2e-9, 0.0]])
    T = np.array([300.5, 299.123456789])
    f2 = tmp_path / "t2.dat"
    sbte.write_tempcell(f2, cen, T, 2, (1e-8, 1e-8, 0.0))
    assert f2.read_text() == "0.5 0.25 300.5\n1 0.2 299.123\n"
    cen3 = np.array([[1e-8, 5e-9, 2.5e-9]])
    f3 = tmp_path / "t3.dat"
    sbte.write_tempcell(f3, cen3, [301.0], 3, (1e-8, 1e-8, 1e-8))
    assert f3.read_text() == "1 0.5 0.25 301\n"
    with pytest.raises(sbte.BteError):
        sbte.write_tempcell(tmp_path / "no" / "such" / "dir.dat", cen, T, 2, (1e-8, 1e-8, 0.0))
