"""MATLAB .mat I/O (multigpugridder_gb300/matio.py): the column-major layout
of the reference's MATLAB arrays against the gridder's [k, j, i] layout, and
round trips."""
import numpy as np
import pytest

scipy_io = pytest.importorskip("scipy.io")

from multigpugridder_gb300.matio import read_mat, write_mat  # noqa: E402


def test_matlab_layout_is_the_gridder_layout(tmp_path):
    # a MATLAB volume V(i, j, k) = i + 10 j + 100 k (0-based), saved as MATLAB would hold it
    nx, ny, nz = 4, 3, 2
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    V = (i + 10 * j + 100 * k).astype(np.float32)              # shape (nx, ny, nz), element [i, j, k]
    axes = np.arange(27, dtype=np.float32).reshape(3, 9)       # 3 directions, 9 floats each
    p = tmp_path / "data.mat"
    scipy_io.savemat(p, {"Volume": V, "coordAxes": np.asfortranarray(axes.T)})
    got = read_mat(p)
    vol = got["Volume"]
    assert vol.shape == (nz, ny, nx) and vol.flags.c_contiguous
    assert vol[1, 2, 3] == 3 + 10 * 2 + 100 * 1                 # [k, j, i]
    # the same bytes as MATLAB's column-major memory
    assert np.array_equal(vol.ravel(), V.ravel(order="F"))
    assert np.array_equal(got["coordAxes"], axes)


def test_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    vol = rng.standard_normal((5, 5, 5)).astype(np.float32)
    imgs = rng.standard_normal((3, 5, 5)).astype(np.float32)
    axes = rng.standard_normal((3, 9)).astype(np.float32)
    p = tmp_path / "rt.mat"
    write_mat(p, Volume=vol, Images=imgs, coordAxes=axes)
    raw = scipy_io.loadmat(p)
    assert raw["Images"].shape == (5, 5, 3) and raw["coordAxes"].shape == (9, 3)
    assert raw["Volume"].dtype == np.float32
    got = read_mat(p)
    assert np.array_equal(got["Volume"], vol)
    assert np.array_equal(got["Images"], imgs)
    assert np.array_equal(got["coordAxes"], axes)
    assert set(read_mat(p, names=["Images"])) == {"Images"}
