import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as g
    return g.load_package()


@pytest.fixture(scope="session")
def lib(pkg):
    return pkg.load_library()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build_port()
    return oracle


@pytest.fixture(scope="session")
def golden_cases():
    """name -> (problem, rhs, params, stored arrays, sha1 of the stored inputs).
    The problem and rhs are the arrays stored in the fixture (the exact inputs
    the reference was run on)."""
    sys.path.insert(0, GOLDEN)
    import make_golden
    geo = make_golden.load_geometry()
    out = {}
    for name, _, _, p in make_golden.cases():
        data = np.load(os.path.join(GOLDEN, name + ".npz"))
        prob = geo.Problem(data["points"], data["normals"], data["weights"], data["curvatures"],
                           hole_centers=data["hole_centers"].reshape(-1, data["points"].shape[1]),
                           hole_start=data["hole_start"], hole_count=data["hole_count"], name=name)
        rhs = data["rhs"]
        out[name] = (prob, rhs, p, data, make_golden.input_hash(prob, rhs))
    return out


@pytest.fixture(scope="session")
def golden_updates():
    """name -> (frames, rhs, params, stored arrays) of the re-factorization
    fixtures: frame 0 is the stored problem, each later frame the one before
    with the stored hole moved by the stored delta (an exact translation);
    rhs (N, 1) serves every frame."""
    sys.path.insert(0, GOLDEN)
    import make_golden
    geo = make_golden.load_geometry()
    out = {}
    for name, _, _, p, _ in make_golden.update_cases():
        data = np.load(os.path.join(GOLDEN, name + ".npz"))
        dim = data["points"].shape[1]
        prob = geo.Problem(data["points"], data["normals"], data["weights"], data["curvatures"],
                           hole_centers=data["hole_centers"].reshape(-1, dim),
                           hole_start=data["hole_start"], hole_count=data["hole_count"], name=name)
        moves = list(zip(data["move_hole"].tolist(), data["move_delta"]))
        out[name] = (make_golden.update_frames(geo, prob, moves), data["rhs"], p, data)
    return out


@pytest.fixture(scope="session")
def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
