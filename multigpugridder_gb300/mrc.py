"""MRC2014 files for volumes and image stacks (host-side I/O).

The reference keeps its data in MATLAB arrays and names .mrc files only in
its .gitignore; this module reads and writes the format cryo-EM data arrive
in, so volumes and images can go to and from the gridder directly.

Layout (MRC2014): a 1024-byte header of 256 little- or big-endian 4-byte
words, an optional extended header of NSYMBT bytes, then the data with x
fastest: a (nz, ny, nx) C-order array here, the gridder's own layout
(vol[k, j, i], i fastest).  Modes read: 0 (int8), 1 (int16), 2 (float32),
6 (uint16), 12 (float16); write: 2 (float32) or 12 (float16).
"""
import struct

import numpy as np

_MODES = {0: np.int8, 1: np.int16, 2: np.float32, 6: np.uint16, 12: np.float16}


def read_mrc(path):
    """(data, voxel_size) of an MRC file; data is (nz, ny, nx) float32 (a stack
    of nz images for a 2-D stack), voxel_size the x cell length / nx in Å."""
    with open(path, "rb") as f:
        head = f.read(1024)
        if len(head) < 1024:
            raise ValueError("%s: shorter than an MRC header" % path)
        # MACHST (word 54): 0x44 0x44 little-endian, 0x11 0x11 big-endian
        endian = ">" if head[212] == 0x11 else "<"
        nx, ny, nz, mode = struct.unpack(endian + "4i", head[0:16])
        if mode not in _MODES:
            raise ValueError("%s: unsupported MRC mode %d" % (path, mode))
        if min(nx, ny, nz) <= 0:
            raise ValueError("%s: invalid dimensions %s" % (path, (nx, ny, nz)))
        mx = struct.unpack(endian + "i", head[28:32])[0]
        cella_x = struct.unpack(endian + "f", head[40:44])[0]
        nsymbt = struct.unpack(endian + "i", head[92:96])[0]
        f.seek(1024 + max(nsymbt, 0))
        dt = np.dtype(_MODES[mode]).newbyteorder(endian)
        count = nx * ny * nz
        data = np.fromfile(f, dtype=dt, count=count)
        if data.size != count:
            raise ValueError("%s: %d values, header says %d" % (path, data.size, count))
    voxel = cella_x / (mx if mx > 0 else nx) if cella_x > 0 else 1.0
    return data.reshape(nz, ny, nx).astype(np.float32), float(voxel)


def write_mrc(path, data, voxel_size=1.0, mode=2):
    """Write a (nz, ny, nx) array (or (ny, nx)) as MRC2014, mode 2 (float32) or
    12 (float16), little-endian, with density statistics and the cell set from
    voxel_size (Å)."""
    if mode not in (2, 12):
        raise ValueError("write_mrc writes mode 2 (float32) or 12 (float16)")
    a = np.asarray(data)
    if a.ndim == 2:
        a = a[None]
    if a.ndim != 3:
        raise ValueError("data must be 2-D or 3-D")
    a = np.ascontiguousarray(a, dtype=_MODES[mode])
    nz, ny, nx = a.shape
    stats = a.astype(np.float64)
    words = bytearray(1024)
    struct.pack_into("<4i", words, 0, nx, ny, nz, mode)
    struct.pack_into("<3i", words, 16, 0, 0, 0)                  # NXSTART, NYSTART, NZSTART
    struct.pack_into("<3i", words, 28, nx, ny, nz)               # MX, MY, MZ
    struct.pack_into("<3f", words, 40, nx * voxel_size, ny * voxel_size, nz * voxel_size)
    struct.pack_into("<3f", words, 52, 90.0, 90.0, 90.0)
    struct.pack_into("<3i", words, 64, 1, 2, 3)                  # MAPC, MAPR, MAPS
    struct.pack_into("<3f", words, 76, float(stats.min()), float(stats.max()), float(stats.mean()))
    struct.pack_into("<i", words, 88, 1 if nz > 1 else 0)        # ISPG: volume, or image stack
    struct.pack_into("<i", words, 92, 0)                         # NSYMBT
    struct.pack_into("<i", words, 108, 20140)                    # NVERSION (word 28)
    words[208:212] = b"MAP "
    words[212:216] = bytes([0x44, 0x44, 0x00, 0x00])            # MACHST: little-endian
    struct.pack_into("<f", words, 216, float(stats.std()))       # RMS
    struct.pack_into("<i", words, 220, 1)                        # NLABL
    label = b"multigpugridder_gb300"
    words[224:224 + len(label)] = label
    with open(path, "wb") as f:
        f.write(bytes(words))
        a.astype(a.dtype.newbyteorder("<")).tofile(f)
