"""BTEcmd, the drop-in for the reference's command-line tool: same flags
(src/BTEMain.cpp:56), the reference's stdout lines, and the --tempcell dump."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form,accel", [("plain", "none"), ("sweep", "none"), ("sweep", "anderson")])
def test_btecmd_2dm2dg(sbte, get_case, tmp_path, form, accel):
    from staticbtesolver_gb300 import _build
    c = get_case("2DM2DG")
    out = tmp_path / "Tempcell.dat"
    cmd = [_build.BTECMD, "-g", c.geo, "-m", c.band, "-b", c.bc, "-d", str(c.DM), "-t", str(c.nt), "-p", str(c.np),
           "-T", "300", "-I", str(c.max_iter), "-x", repr(c.L[0]), "-y", repr(c.L[1]), "--form", form,
           "--accel", accel, "--tempcell", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    margins = [float(m) for m in re.findall(r"Iteration #\d+\t Margin per band per cell: (\S+)", r.stdout)]
    if accel == "none":
        assert len(margins) == int(c.ref["n_iter"])
    else:  # the accelerated iteration stops at the same margin, sooner
        assert len(margins) < int(c.ref["n_iter"]) and margins[-1] <= 1e-5
    q = {int(k): float(v) for k, v in re.findall(r"heat flux of Boundary Condition #(\d+): (\S+)", r.stdout)}
    q = np.array([q[k] for k in sorted(q)])
    big = np.abs(c.ref["q"]) > 1e-3 * np.abs(c.ref["q"]).max()
    # the printed fluxes carry 6 significant digits
    np.testing.assert_allclose(q[big], c.ref["q"][big], rtol=6e-6 if accel == "none" else 1e-4)
    assert re.search(r"N_cell: \d+", r.stdout) and "Time taken by iteration" in r.stdout
    rows = np.loadtxt(out)
    assert rows.shape == (c.ref["T"].size, 3)
    assert np.abs(rows[:, 2] - c.ref["T"]).max() <= 6e-4  # printed to 6 significant digits
    assert rows[:, :2].min() >= 0.0 and rows[:, :2].max() <= 1.0  # centroids / L


def test_btecmd_dsa_diffusive(tmp_path):
    """--dsa on the diffusive 12x12 square of tests/golden/diffusive: the
    flag reaches the solver (a few tens of outer iterations instead of the
    reference's thousands) and the stop is the reference's margin test; the
    printed fluxes are those of the iteration's fixed point."""
    import json

    from conftest import GOLDEN
    from staticbtesolver_gb300 import _build
    d = os.path.join(GOLDEN, "diffusive", "square12_b8")
    meta = json.load(open(os.path.join(d, "expected.json")))
    ref = dict(np.load(os.path.join(d, "ref.npz")))
    cmd = [_build.BTECMD, "-g", os.path.join(d, "mesh.mphtxt"), "-m", os.path.join(d, "band.dat"), "-b",
           os.path.join(d, "inputbc.dat"), "-d", str(meta["DM"]), "-t", str(meta["num_theta"]), "-p",
           str(meta["num_phi"]), "-T", "300", "-I", "200", "-x", repr(meta["side"]), "-y", repr(meta["side"]),
           "--form", "sweep", "--dsa"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    margins = [float(m) for m in re.findall(r"Iteration #\d+\t Margin per band per cell: (\S+)", r.stdout)]
    assert 0 < len(margins) <= 30 and margins[-1] <= 1e-5 and all(m > 1e-5 for m in margins[:-1])
    q = {int(k): float(v) for k, v in re.findall(r"heat flux of Boundary Condition #(\d+): (\S+)", r.stdout)}
    q = np.array([q[k] for k in sorted(q)])
    big = np.abs(ref["q_fixed"]) > 1e-3 * np.abs(ref["q_fixed"]).max()
    np.testing.assert_allclose(q[big], ref["q_fixed"][big], rtol=1e-4)
