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
