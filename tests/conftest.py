"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; everything else runs on CPU."""
import gzip
import json
import os
import shutil
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)

TESTSH_CASES = ["2DM1DG", "3DM1DG", "2DM2DG", "3DM2DG", "3DM3DG"]
SYNTH_CASES = ["square10_b40", "cube4_b2", "slab1d", "square16_b8"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: takes more than ~30 s")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def sbte():
    import staticbtesolver_gb300 as S
    S.build()
    return S


class Case:
    """One golden case: input files, solver parameters and expected values."""

    def __init__(self, name, tmpdir):
        self.name = name
        if name in SYNTH_CASES:
            d = os.path.join(GOLDEN, "synth", name)
            meta = json.load(open(os.path.join(d, "expected.json")))
            geo = meta["geo"]
            self.geo = os.path.join(d, geo) if geo.endswith(".mphtxt") else geo
            self.bc, self.band = os.path.join(d, meta["bc_file"]), os.path.join(d, meta["band_file"])
        else:
            d = os.path.join(GOLDEN, name)
            meta = json.load(open(os.path.join(d, "expected.json")))
            if name in ("2Dcase2", "2Dcase5"):
                self.geo = os.path.join(tmpdir, f"{name}.mphtxt")
                if not os.path.exists(self.geo):
                    with gzip.open(os.path.join(d, "mesh.mphtxt.gz"), "rb") as fi, open(self.geo, "wb") as fo:
                        shutil.copyfileobj(fi, fo)
            else:
                geo = meta["geo"]
                self.geo = os.path.join(d, geo) if geo.endswith(".mphtxt") else geo
            self.bc, self.band = os.path.join(d, "inputbc.dat"), os.path.join(d, "band.dat")
        self.meta = meta
        self.DM, self.nt, self.np = meta["DM"], meta["num_theta"], meta["num_phi"]
        self.L = (meta["L_x"], meta["L_y"], meta["L_z"])
        self.T_ref = meta.get("T_ref", 300.0)
        self.max_iter = meta["max_iter"]
        self.ref = dict(np.load(os.path.join(d, "ref.npz")))

    def args(self):
        return (self.geo, self.bc, self.band, self.DM, self.nt, self.np, self.T_ref, *self.L)


@pytest.fixture(scope="session")
def case_dir(tmp_path_factory):
    return str(tmp_path_factory.mktemp("cases"))


@pytest.fixture(scope="session")
def get_case(case_dir):
    cache = {}

    def _get(name):
        if name not in cache:
            cache[name] = Case(name, case_dir)
        return cache[name]

    return _get


def rel_l2(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
