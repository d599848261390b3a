"""Reading and writing problems in the reference's text format
(psba_gb300.io).  A round trip through the files keeps the residuals; the
reference's own example files load and the oracle solves them (where the
reference's sources are present; they are read in place, never copied)."""
import os

import numpy as np
import pytest

import oracle
from psba_gb300 import io as pio
from psba_gb300 import scenes

REF_DATA = "/root/reference/data"


@pytest.mark.parametrize("cnp", [6, 11, 16])
def test_round_trip_keeps_residuals(tmp_path, cnp):
    sc = scenes.arc_scene(seed=2, n_cams=6, n_pts=150)
    if cnp > 6:
        sc = scenes.with_intrinsics(sc, cnp, seed=3)
    # move the cameras off v = 0 so that the composed rotation is written
    rng = np.random.default_rng(0)
    cams = sc.cams.copy()
    cams[:, :3] = rng.normal(0.0, 0.01, size=(sc.n_cams, 3))
    cov = np.tile(np.array([[0.25, 0.01], [0.01, 0.36]]), (sc.n_obs, 1, 1))
    pio.write_scene(tmp_path / "c.txt", tmp_path / "p.txt", sc, cams=cams, cov=cov)
    back = pio.load_scene(tmp_path / "c.txt", tmp_path / "p.txt", cnp=cnp)
    assert back.n_cams == sc.n_cams and back.n_pts == sc.n_pts and back.n_obs == sc.n_obs
    assert np.array_equal(back.obs_pt, sc.obs_pt) and np.array_equal(back.obs_cam, sc.obs_cam)
    assert np.array_equal(back.meas, sc.meas) and np.array_equal(back.pts, sc.pts)
    assert np.allclose(back.cov, cov)
    assert np.all(back.cams[:, :3] == 0.0)
    e0 = oracle.residual(oracle.OracleProblem(sc), cams, sc.pts)
    ew = oracle.residual(oracle.OracleProblem(back), back.cams, back.pts)  # whitened by back.cov
    plain = back.copy()
    plain.cov = None
    e1 = oracle.residual(oracle.OracleProblem(plain), back.cams, back.pts)
    assert np.abs(e0 - e1).max() <= 1e-8
    L = oracle.whitening(cov)
    assert np.allclose(ew[:, 0], L[:, 0] * e1[:, 0] + L[:, 1] * e1[:, 1], rtol=1e-12, atol=1e-12)
    assert np.allclose(ew[:, 1], L[:, 2] * e1[:, 1], rtol=1e-12, atol=1e-12)
    Lm = np.zeros((sc.n_obs, 2, 2))
    Lm[:, 0, 0], Lm[:, 0, 1], Lm[:, 1, 1] = L[:, 0], L[:, 1], L[:, 2]
    assert np.allclose(np.einsum("oki,okj->oij", Lm, Lm) @ cov, np.eye(2), atol=1e-12)


def test_reader_sorts_frames_and_rejects_repeats(tmp_path):
    (tmp_path / "c.txt").write_text("# two cameras\n" + "800 320 240 1 0  1 0 0 0  0 0 0\n" * 2)
    (tmp_path / "p.txt").write_text("0 0 5  2  1 321.0 240.5  0 319.5 239.0\n0.1 0 5  1  0 330 240\n")
    sc = pio.load_scene(tmp_path / "c.txt", tmp_path / "p.txt")
    assert list(sc.obs_pt) == [0, 0, 1] and list(sc.obs_cam) == [0, 1, 0]
    assert sc.meas[0].tolist() == [319.5, 239.0]
    (tmp_path / "p2.txt").write_text("0 0 5  2  1 321.0 240.5  1 319.5 239.0\n")
    with pytest.raises(ValueError):
        pio.load_scene(tmp_path / "c.txt", tmp_path / "p2.txt")
    (tmp_path / "p3.txt").write_text("0 0 5  1  2 321.0 240.5\n")
    with pytest.raises(ValueError):
        pio.load_scene(tmp_path / "c.txt", tmp_path / "p3.txt")
    (tmp_path / "c2.txt").write_text("1 0 0 0 0 0\n")
    with pytest.raises(ValueError):
        pio.read_cameras(tmp_path / "c2.txt")


@pytest.mark.skipif(not os.path.isdir(REF_DATA), reason="reference example files not present")
@pytest.mark.parametrize("cams,pts,cnp", [("7camsvarK.txt", "7pts.txt", 6), ("7camsvarK.txt", "7pts.txt", 11),
                                          ("54camsvarKD.txt", "54pts.txt", 16)])
def test_reference_example_files_load_and_solve(cams, pts, cnp):
    sc = pio.load_scene(os.path.join(REF_DATA, cams), os.path.join(REF_DATA, pts), cnp=cnp)
    assert sc.n_obs > 0 and np.all(np.isfinite(sc.meas))
    r = oracle.levmar(sc, allow_switch=0, max_iter=20)
    assert np.isfinite(r.final_cost) and r.final_cost < r.initial_cost
