import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a GPU and the built CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def avatar():
    from insta_gb300 import synthetic as S
    return S.make_avatar(0)


@pytest.fixture(scope="session")
def frame0(avatar):
    return avatar.frame(avatar.frame_coeffs(0))


@pytest.fixture(scope="session")
def oracle_frame(oracle, avatar, frame0):
    """Oracle triangles, adjacency and BVH for frame 0."""
    can = oracle.build_triangles(avatar.canonical, None, avatar.faces, avatar.mask)
    dtr = oracle.build_triangles(frame0, avatar.canonical, avatar.faces, avatar.mask)
    adj = oracle.adjacency(avatar.faces, avatar.n_verts)
    bvh = oracle.Bvh(dtr)
    return {"can": can, "def": dtr, "adj": adj, "bvh": bvh}


@pytest.fixture(scope="session")
def ctx():
    from insta_gb300 import abi
    c = abi.Context(0)
    yield c
    c.close()


def psnr(a, b, peak=1.0):
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)
