"""MATLAB .mat files (format v5) for the arrays the reference's MATLAB class
holds (host-side I/O).

The reference keeps its data in MATLAB arrays (MultiGPUGridder_Matlab_Class.m:
27-31: coordAxes 9 x NumAxes, Volume N x N x N, Images N x N x n, CASVolume
V x V x V, CASImages M x M x n, all single) and lists *.mat files in its
.gitignore.  MATLAB stores arrays column-major, so V(i, j, k) sits at flat
offset i + j*N + k*N*N, which is the gridder's own layout read as a C-order
[k, j, i] array.  These helpers convert between the two: a 3-D MATLAB array of
shape (nx, ny, nz) becomes a (nz, ny, nx) float32 array, a 2-D image (nx, ny)
becomes (ny, nx), and coordAxes (9 x n) becomes (n, 9) -- and back on writing.

Format v5 only (scipy.io); v7.3 files are HDF5 and need h5py.
"""
import numpy as np

AXES_NAMES = ("coordAxes",)


def _from_matlab(name, a):
    a = np.asarray(a)
    if a.dtype.kind not in "fiub":
        return a
    if name in AXES_NAMES or (a.ndim == 2 and a.shape[0] == 9 and name.lower().endswith("axes")):
        return np.ascontiguousarray(np.asarray(a, np.float32).reshape(9, -1, order="F").T)
    if a.ndim in (2, 3):
        return np.ascontiguousarray(np.asarray(a, np.float32).transpose(tuple(range(a.ndim))[::-1]))
    return np.asarray(a, np.float32)


def _to_matlab(name, a):
    a = np.asarray(a, np.float32)
    if name in AXES_NAMES:
        return np.asfortranarray(a.reshape(-1, 9).T)
    if a.ndim in (2, 3):
        return np.asfortranarray(a.transpose(tuple(range(a.ndim))[::-1]))
    return a


def read_mat(path, names=None):
    """Arrays of a v5 .mat file in the gridder's layout, as a dict name ->
    float32 array (numeric variables only; `names` selects some)."""
    from scipy.io import loadmat

    d = loadmat(path)
    out = {}
    for k, v in d.items():
        if k.startswith("__") or (names is not None and k not in names):
            continue
        if isinstance(v, np.ndarray) and v.dtype.kind in "fiub":
            out[k] = _from_matlab(k, v)
    return out


def write_mat(path, **arrays):
    """Write gridder-layout arrays as MATLAB single arrays (v5): 3-D
    [k, j, i] -> nx x ny x nz, 2-D [j, i] -> nx x ny, coordAxes (n, 9) -> 9 x n."""
    from scipy.io import savemat

    savemat(path, {k: _to_matlab(k, v) for k, v in arrays.items()}, format="5", do_compression=False)
