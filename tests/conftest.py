import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    from psba_gb300 import scenes
    z = np.load(os.path.join(ROOT, "tests", "golden", "ref_arc7.npz"))
    sc = scenes.Scene("golden", z["K"], z["q0"], z["cams"], z["pts"], z["meas"], z["obs_pt"], z["obs_cam"])
    return sc, z


REF_DATA_NAMES = ("7cams", "54cams", "trafalgar21")


@pytest.fixture(scope="session")
def ref_data():
    """The reference's example problems (data/7camsvarK+7pts, 54camsvarK+54pts,
    Trafalgar-21-11315), as tests/golden/make_fixtures.py parsed them."""
    import numpy as np
    from psba_gb300 import scenes
    z = np.load(os.path.join(ROOT, "tests", "golden", "ref_data.npz"))
    out = {}
    for n in REF_DATA_NAMES:
        out[n] = scenes.Scene(n, z[n + "_K"], z[n + "_q0"], z[n + "_cams"], z[n + "_pts"], z[n + "_meas"],
                              z[n + "_obs_pt"], z[n + "_obs_cam"])
    return out
