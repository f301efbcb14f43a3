"""Failure paths of the C ABI: the reference prints a message and exit(1)s
(src/StaticBTESolver.cpp:218-219, 244-246, 254-255, 429-430); here every such
case returns a status and leaves the context usable.  Host-side checks only:
nothing here faults, traps or hangs a GPU."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx(sbte, get_case, name="square10_b40"):
    c = get_case(name)
    p = sbte.Problem(*c.args())
    return c, p, p.arrays(), sbte.Context(0)


def test_non_finite_band_data_is_numerical(sbte, get_case):
    c, p, a, ctx = _ctx(sbte, get_case)
    ctx.set_arrays(a)
    L, _ = sbte._load()
    b = a["bands"]
    for key, bad in (("vg", np.nan), ("tau", np.inf), ("C", -np.inf), ("Lr", np.nan)):
        arr = {k: np.array(v, float) for k, v in b.items()}
        arr[key][1] = bad
        st = L.bte_set_bands(ctx._h, len(arr["vg"]), arr["vg"], arr["tau"], arr["C"], arr["Lr"])
        assert st == 7, key
        assert b"non-finite" in L.bte_last_error(ctx._h)
    # the good bands are still there: the context solves as before
    st, rep = ctx.solve(max_iter=c.max_iter, tol=1e-5, form=sbte.FORM_SWEEP)
    assert st == 0 and rep.n_iter == int(c.ref["n_iter"])
    ctx.close()


def test_boundary_type_unsupported_for_mesh_dimension(sbte, get_case):
    """Specular type 33 (z mirror) on a 2D mesh: the reference exit(1)s (:244-246)."""
    c, p, a, ctx = _ctx(sbte, get_case)
    bcs = dict(a["bcs"])
    bcs["type"] = np.array(bcs["type"]).copy()
    bcs["type"][1] = 33
    ctx.set_arrays(dict(a, bcs=bcs))
    with pytest.raises(sbte.BteError) as e:
        ctx.solve(max_iter=5, form=sbte.FORM_SWEEP)
    assert e.value.status == 5
    bcs["type"][1] = 7  # no such type at all
    ctx.set_arrays(dict(a, bcs=bcs))
    with pytest.raises(sbte.BteError) as e:
        ctx.solve(max_iter=5)
    assert e.value.status == 5
    ctx.set_arrays(a)  # a valid set again solves
    st, rep = ctx.solve(max_iter=c.max_iter, tol=1e-5, form=sbte.FORM_SWEEP)
    assert st == 0
    ctx.close()


def test_corrupt_neighbour_index_is_rejected(sbte, get_case):
    c, p, a, ctx = _ctx(sbte, get_case)
    L, _ = sbte._load()
    nbr = np.ascontiguousarray(a["nbr"], np.int32).ravel().copy()
    f64 = lambda x: np.ascontiguousarray(x, np.float64).ravel()
    for bad in (a["n_cell"], a["n_cell"] + 1000, 2 ** 30):
        nb = nbr.copy()
        nb[7] = bad
        st = L.bte_set_geometry(ctx._h, a["dim"], a["n_cell"], a["n_face"], nb, f64(a["area"]), f64(a["normal"]),
                                f64(a["volume"]))
        assert st == 1
        assert b"out of range" in L.bte_last_error(ctx._h)
    # wrong face count for the dimension, and a non-finite normal
    st = L.bte_set_geometry(ctx._h, a["dim"], a["n_cell"], a["n_face"] + 1, nbr, f64(a["area"]), f64(a["normal"]),
                            f64(a["volume"]))
    assert st == 1
    nrm = f64(a["normal"]).copy()
    nrm[4] = np.nan
    st = L.bte_set_geometry(ctx._h, a["dim"], a["n_cell"], a["n_face"], nbr, f64(a["area"]), nrm, f64(a["volume"]))
    assert st == 1
    # solving before any geometry was accepted is a state error
    with pytest.raises(sbte.BteError) as e:
        ctx.solve(max_iter=2)
    assert e.value.status == 2
    ctx.close()


def test_inner_iteration_limit_is_counted_not_fatal(sbte, get_case):
    """inner_maxit = 1: no system converges; the reference would carry on with
    the last iterates, and so does this path, counting them."""
    c, p, a, ctx = _ctx(sbte, get_case)
    ctx.set_arrays(a)
    st, rep = ctx.solve(max_iter=2, tol=1e-5, form=sbte.FORM_PLAIN, inner_maxit=1)
    assert st == 6  # not converged: max_iter reached
    assert rep.inner_unconverged > 0 and rep.inner_solves == 2 * p.n_dir * p.n_band
    st, rep = ctx.solve(max_iter=2, tol=1e-5, form=sbte.FORM_SWEEP, inner_maxit=1)
    assert st == 6 and rep.inner_unconverged == 0  # acyclic: one sweep is exact
    ctx.close()


def test_bad_options_are_rejected(sbte, get_case):
    c, p, a, ctx = _ctx(sbte, get_case)
    ctx.set_arrays(a)
    for kw in (dict(inner_maxit=0), dict(inner_tol=0.0), dict(form=9), dict(accel=5), dict(accel=3, accel_every=9),
               dict(dsa=True, dsa_tol=-1.0)):
        with pytest.raises(sbte.BteError) as e:
            ctx.solve(max_iter=2, **kw)
        assert e.value.status == 1, kw
    ctx.close()


def test_dsa_rejects_1d_meshes(sbte, get_case):
    c, p, a, ctx = _ctx(sbte, get_case, "slab1d")
    ctx.set_arrays(a)
    with pytest.raises(sbte.BteError) as e:
        ctx.solve(max_iter=2, dsa=True)
    assert e.value.status == 1
    ctx.close()
