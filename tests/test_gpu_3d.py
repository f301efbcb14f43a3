"""3D: tetrahedral meshes, DM=3, 128 directions, x-faces isothermal, y/z faces
specular (types 32/33).  Mid-size parity against the oracle computed here;
the full-size cube200k workload (196,608 tets x 5,120 systems) by properties
that hold at any size."""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cube6(tmp_path_factory):
    from staticbtesolver_gb300 import synth
    return synth.make_problem("cube6_b8", str(tmp_path_factory.mktemp("cube6")))


def _args(p):
    return (p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)


def _solve(sbte, args, **kw):
    prob = sbte.Problem(*args)
    ctx = sbte.Context(0).load(prob)
    st, rep = ctx.solve(**kw)
    res = ctx.result(st, rep)
    ctx.close()
    return res


@pytest.mark.parametrize("form_name", ["FORM_SWEEP", "FORM_PLAIN"])
def test_cube_matches_oracle(sbte, oracle_mod, cube6, form_name):
    o = oracle_mod.Oracle(*_args(cube6)).run(max_iter=1000, outer_tol=1e-5, threads=os.cpu_count() or 1)
    res = _solve(sbte, _args(cube6), max_iter=1000, tol=1e-5, form=getattr(sbte, form_name))
    assert res.status == 0
    assert res.report["n_iter"] == o.n_iter
    assert rel_l2(res.T - 300, o.T - 300) < 1e-6
    big = np.abs(o.q) > 1e-3 * np.abs(o.q).max()
    np.testing.assert_allclose(res.q[big], o.q[big], rtol=1e-6)


def test_cube200k_full_size_properties(sbte, tmp_path):
    from staticbtesolver_gb300 import synth
    p = synth.make_problem("cube200k", str(tmp_path))
    a = _solve(sbte, _args(p), max_iter=1000, tol=1e-5, form=sbte.FORM_SWEEP)
    assert a.status == 0 and a.report["converged"]
    assert a.report["inner_iterations"] == a.report["inner_solves"]  # acyclic: one sweep per system
    # maximum principle: the field stays between the wall temperatures
    assert a.T.min() > 299.0 - 1e-9 and a.T.max() < 301.0 + 1e-9
    # the two isothermal faces carry opposite fluxes (entities 0 and 5 are rows 0 and 1)
    assert a.q[0] < 0 < a.q[1]
    assert abs(a.q[0] + a.q[1]) < 0.02 * abs(a.q[0])
    # bitwise reproducible
    b = _solve(sbte, _args(p), max_iter=1000, tol=1e-5, form=sbte.FORM_SWEEP)
    np.testing.assert_array_equal(a.T, b.T)
