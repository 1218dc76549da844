"""MRC2014 I/O (multigpugridder_gb300/mrc.py): round trips in both written
modes, the header words other software reads, big-endian files and the
integer modes, and an extended header that is skipped."""
import struct

import numpy as np
import pytest

from multigpugridder_gb300.mrc import read_mrc, write_mrc


def test_round_trip_volume_and_header(tmp_path):
    rng = np.random.default_rng(0)
    vol = rng.standard_normal((6, 5, 4)).astype(np.float32)
    p = tmp_path / "v.mrc"
    write_mrc(p, vol, voxel_size=1.5)
    got, vs = read_mrc(p)
    assert np.array_equal(got, vol) and vs == 1.5
    with open(p, "rb") as f:
        head = f.read(1024)
    assert struct.unpack("<4i", head[:16]) == (4, 5, 6, 2)          # NX NY NZ MODE, x fastest
    assert struct.unpack("<3i", head[28:40]) == (4, 5, 6)           # MX MY MZ
    assert struct.unpack("<3f", head[40:52]) == (6.0, 7.5, 9.0)     # cell (Å)
    assert struct.unpack("<3i", head[64:76]) == (1, 2, 3)           # MAPC MAPR MAPS
    assert head[208:212] == b"MAP " and head[212:214] == b"\x44\x44"
    assert struct.unpack("<i", head[108:112])[0] == 20140
    dmin, dmax, dmean = struct.unpack("<3f", head[76:88])
    assert np.isclose(dmin, vol.min()) and np.isclose(dmax, vol.max()) and np.isclose(dmean, vol.mean())
    assert p.stat().st_size == 1024 + vol.nbytes


def test_round_trip_float16_and_2d(tmp_path):
    img = np.linspace(-2, 2, 12, dtype=np.float32).reshape(3, 4)
    p = tmp_path / "i.mrc"
    write_mrc(p, img, mode=12)
    got, _ = read_mrc(p)
    assert got.shape == (1, 3, 4)
    assert np.array_equal(got[0], img.astype(np.float16).astype(np.float32))


@pytest.mark.parametrize("mode,dt", [(0, np.int8), (1, np.int16), (6, np.uint16), (2, np.float32)])
def test_reads_other_modes_big_endian_and_extended_header(tmp_path, mode, dt):
    data = (np.arange(2 * 3 * 4) % 50).astype(dt).reshape(2, 3, 4)
    head = bytearray(1024)
    struct.pack_into(">4i", head, 0, 4, 3, 2, mode)
    struct.pack_into(">3i", head, 28, 4, 3, 2)
    struct.pack_into(">3f", head, 40, 8.0, 6.0, 4.0)
    struct.pack_into(">i", head, 92, 80)                             # NSYMBT: 80 bytes to skip
    head[208:212] = b"MAP "
    head[212:216] = bytes([0x11, 0x11, 0, 0])                        # big-endian
    p = tmp_path / "b.mrc"
    with open(p, "wb") as f:
        f.write(bytes(head) + b"\x07" * 80 + data.astype(np.dtype(dt).newbyteorder(">")).tobytes())
    got, vs = read_mrc(p)
    assert np.array_equal(got, data.astype(np.float32)) and vs == 2.0


def test_rejects_bad_files(tmp_path):
    p = tmp_path / "short.mrc"
    p.write_bytes(b"\x00" * 100)
    with pytest.raises(ValueError):
        read_mrc(p)
    head = bytearray(1024)
    struct.pack_into("<4i", head, 0, 2, 2, 2, 4)                     # mode 4 (complex) unsupported
    p2 = tmp_path / "m4.mrc"
    p2.write_bytes(bytes(head) + b"\x00" * 64)
    with pytest.raises(ValueError):
        read_mrc(p2)
