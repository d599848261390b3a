"""Reading and writing problems in the reference's text format
(psba_gb300.io).  A round trip through the files keeps the residuals; the
reference's own example files load and the oracle solves them, and the
reader agrees bit for bit with the reference's own reader
(readInitialSBAEstimate, PSBA/readparams.cpp:444-519, compiled here from
the reference's sources into oracle/_ref) on every array main() takes from
it (PSBA/main.cpp:102-149).  Those checks run where the reference checkout
is present; tests/golden/ref_data.npz carries the parsed files elsewhere.
"""
import os

import numpy as np
import pytest

import oracle
from oracle import build as oracle_build
from psba_gb300 import io as pio
from psba_gb300 import scenes

REF_DATA = oracle_build.reference_data_dir()
needs_reference = pytest.mark.skipif(REF_DATA is None, reason="reference example files not present")


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


@needs_reference
@pytest.mark.parametrize("cams,pts,cnp", [("7camsvarK.txt", "7pts.txt", 6), ("7camsvarK.txt", "7pts.txt", 11),
                                          ("54camsvarKD.txt", "54pts.txt", 16)])
def test_reference_example_files_load_and_solve(cams, pts, cnp):
    sc = pio.load_scene(os.path.join(REF_DATA, cams), os.path.join(REF_DATA, pts), cnp=cnp)
    assert sc.n_obs > 0 and np.all(np.isfinite(sc.meas))
    r = oracle.levmar(sc, allow_switch=0, max_iter=20)
    assert np.isfinite(r.final_cost) and r.final_cost < r.initial_cost


# the files of tests/golden/make_fixtures.py, and the counts they hold
FIXTURE_FILES = {"7cams": ("7camsvarK.txt", "7pts.txt", 7, 465, 1916),
                 "54cams": ("54camsvarK.txt", "54pts.txt", 54, 5207, 24609),
                 "trafalgar21": ("Trafalgar-21-11315-cams.txt", "Trafalgar-21-11315-pts.txt", 21, 11315, 36455)}


@needs_reference
@pytest.mark.parametrize("name", sorted(FIXTURE_FILES) + ["54camsKD"])
def test_reader_matches_the_reference_reader(name):
    from oracle import ref
    if not ref.reader_available():
        pytest.skip("reference reader not built")
    if name == "54camsKD":
        cams, pts, cnp, filecnp = "54camsvarKD.txt", "54pts.txt", 16, 17
    else:
        cams, pts = FIXTURE_FILES[name][:2]
        cnp, filecnp = 11, 12  # PSBA/main.cpp:73,102-110
    ms, initrot, imgpts, cov, vmask = ref.read_sba(os.path.join(REF_DATA, cams), os.path.join(REF_DATA, pts),
                                                   cnp=cnp, filecnp=filecnp)
    sc = pio.load_scene(os.path.join(REF_DATA, cams), os.path.join(REF_DATA, pts), cnp=6 if cnp == 11 else 16)
    C = sc.n_cams
    m = ms[:C * cnp].reshape(C, cnp)
    # main.cpp:131-149: the rotation's vector part is zeroed, K split off, the
    # file's rotation kept in initrot
    assert np.array_equal(m[:, :5], sc.K)
    assert np.array_equal(initrot.reshape(C, 4), sc.q0)
    assert np.array_equal(m[:, cnp - 3:], sc.cams[:, 3:6])
    assert np.all(sc.cams[:, :3] == 0.0)
    if cnp == 16:
        assert np.array_equal(m[:, :5], sc.cams[:, 6:11]) and np.array_equal(m[:, 5:10], sc.cams[:, 11:16])
    assert np.array_equal(ms[C * cnp:].reshape(-1, 3), sc.pts)
    # generate_idxs (misc.cpp:189-197) orders observations point-major by the
    # visibility mask; the files list frames in ascending order, so imgpts'
    # file order is that order
    obs = np.argwhere(vmask == 1)
    assert np.array_equal(obs[:, 0], sc.obs_pt) and np.array_equal(obs[:, 1], sc.obs_cam)
    assert np.array_equal(imgpts.reshape(-1, 2), sc.meas)
    assert cov is None and sc.cov is None


@needs_reference
@pytest.mark.parametrize("name", sorted(FIXTURE_FILES))
def test_committed_fixture_is_the_reference_file(name, ref_data):
    cams, pts, n_cams, n_pts, n_obs = FIXTURE_FILES[name]
    sc = pio.load_scene(os.path.join(REF_DATA, cams), os.path.join(REF_DATA, pts), cnp=6)
    z = ref_data[name]
    assert (z.n_cams, z.n_pts, z.n_obs) == (n_cams, n_pts, n_obs)
    for k in ("K", "q0", "cams", "pts", "meas", "obs_pt", "obs_cam"):
        assert np.array_equal(getattr(z, k), getattr(sc, k)), k


@pytest.mark.parametrize("name", sorted(FIXTURE_FILES))
def test_fixture_counts_and_oracle_solve(name, ref_data):
    sc = ref_data[name]
    assert (sc.n_cams, sc.n_pts, sc.n_obs) == FIXTURE_FILES[name][2:]
    r = oracle.levmar(sc, allow_switch=0, max_iter=5)
    assert np.isfinite(r.final_cost) and r.final_cost < r.initial_cost
