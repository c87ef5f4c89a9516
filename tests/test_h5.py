"""HDF5 input and output without libhdf5 (include/e3d_micro.h, csrc/h5lite.cpp),
CPU only.

- A file written by the HDF5 library itself -- MATLAB 7.4's -v7.3 MAT-file that
  SciPy ships as test data (user block, version-0 superblock, attributes on
  every dataset) -- is read back: "testdouble" holds 0:pi/4:2*pi.
- Microstructure files (the reference's MATLAB generator's layout,
  src/microstructure_gen.m:876-889) and fullfield_poly.h5 (src/elas3dxtal_pcg.f90:
  2840-2874) round-trip through the writer and the reader, with the reference's
  checks on the input (:2939-2942, :2966-2969, :2986-2989).
- Structures the writer does not produce but the HDF5 library may: an object
  header continued in a second block, big-endian integers; and ones the reader
  refuses: chunked storage, a newer superblock, a file that is not HDF5.
"""
import glob
import os
import struct

import numpy as np
import pytest

import elas3d_xtal_gb300 as e3d
from elas3d_xtal_gb300 import workloads as W


def _matlab_file():
    import scipy

    hits = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data",
                                  "testhdf5_7.4_GLNX86.mat"))
    return hits[0] if hits else None


def test_reads_a_file_written_by_the_hdf5_library():
    path = _matlab_file()
    if path is None:
        pytest.skip("SciPy's HDF5 MAT-file test data is not installed")
    with open(path, "rb") as f:
        assert f.read(1024)[512:520] == b"\x89HDF\r\n\x1a\n"  # superblock after a 512-byte user block
    v = e3d.h5_read(path, "testdouble")
    assert v.shape == (9, 1)  # MATLAB's 1 x 9 row, dimensions reversed
    assert np.allclose(v.ravel(), np.arange(9) * np.pi / 4, rtol=0, atol=1e-15)


def test_micro_round_trip_and_layout(tmp_path):
    p, pix, rod = W.c2(n=18)
    path = str(tmp_path / "input_structure_poly.h5")
    e3d.h5_micro_write(path, pix, rod, (18, 18, 18))
    npix, nori, dims = e3d.h5_micro_info(path)
    assert (npix, nori, dims) == (p.ns, rod.size, (18, 18, 18))
    q, r = e3d.h5_micro_read(path, p.ns, p.nphase - 1)
    assert np.array_equal(q, pix) and np.array_equal(r, rod)
    assert e3d.h5_read(path, "pix").shape == (1, p.ns)  # an N x 1 MATLAB column
    assert e3d.h5_read(path, "orientation").shape == (1, rod.size)
    with open(path, "rb") as f:
        head = f.read(96)
    assert head[:8] == b"\x89HDF\r\n\x1a\n" and head[8] == 0  # version-0 superblock
    assert struct.unpack_from("<Q", head, 40)[0] == os.path.getsize(path)  # end-of-file address


def test_micro_read_applies_the_reference_checks(tmp_path):
    p, pix, rod = W.c2(n=10)
    ng = p.nphase - 1
    path = str(tmp_path / "m.h5")
    e3d.h5_micro_write(path, pix, rod, (10, 10, 10))
    with pytest.raises(ValueError, match="does not match simulation ns"):
        e3d.h5_micro_read(path, p.ns + 1, ng)
    with pytest.raises(ValueError, match="orientation size"):
        e3d.h5_micro_read(path, p.ns, ng + 1)
    bad = pix.copy()
    bad[123] = ng + 2
    e3d.h5_micro_write(path, bad, rod, (10, 10, 10))
    with pytest.raises(ValueError, match="out of bounds"):
        e3d.h5_micro_read(path, p.ns, ng)
    bad[123] = 0
    e3d.h5_micro_write(path, bad, rod, (10, 10, 10))
    with pytest.raises(ValueError, match="out of bounds"):
        e3d.h5_micro_read(path, p.ns, ng)
    with pytest.raises(OSError):
        e3d.h5_micro_read(str(tmp_path / "missing.h5"), p.ns, ng)
    junk = tmp_path / "junk.h5"
    junk.write_bytes(b"not an HDF5 file" * 64)
    with pytest.raises(ValueError, match="not an HDF5 file"):
        e3d.h5_micro_read(str(junk), p.ns, ng)


def test_fullfield_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    ns = 7 * 5 * 4
    pix = rng.integers(1, 5, size=ns).astype(np.int32)
    vm = rng.random(ns) * 1e8
    sigma = rng.normal(size=6 * ns) * 1e8
    path = str(tmp_path / "fullfield_poly.h5")
    e3d.h5_fullfield_write(path, pix, vm, sigma)
    assert np.array_equal(e3d.h5_read(path, "pix"), pix)
    assert np.array_equal(e3d.h5_read(path, "vm"), vm)
    st = e3d.h5_read(path, "stress_tensor")
    assert st.shape == (6, ns)  # the Fortran writer's (ns, 6), reversed in the file
    assert np.array_equal(st.ravel(), sigma)


# ---- byte-level variants of a written file -------------------------------
def _object_headers(buf):
    """(name, header address, header length) of every dataset, found through
    the one symbol-table node the writer makes."""
    i = buf.index(b"SNOD")
    nsym = struct.unpack_from("<H", buf, i + 6)[0]
    heap = buf.index(b"HEAP")
    heap_data = struct.unpack_from("<Q", buf, heap + 24)[0]
    out = []
    for s in range(nsym):
        noff, oh = struct.unpack_from("<QQ", buf, i + 8 + 40 * s)
        name = buf[heap_data + noff: buf.index(b"\0", heap_data + noff)].decode()
        out.append((name, oh, struct.unpack_from("<I", buf, oh + 8)[0]))
    return out


def _messages(buf, oh, length):
    q, out = oh + 16, []
    while q + 8 <= oh + 16 + length:
        t, sz = struct.unpack_from("<HH", buf, q)
        out.append((t, q, sz))
        q += 8 + sz
    return out


def test_object_header_continuation_is_followed(tmp_path):
    """Moves the attribute of "pix" into a continuation block at the end of the
    file, as the HDF5 library does when a header outgrows its first block."""
    p, pix, rod = W.c2(n=12)
    path = tmp_path / "c.h5"
    e3d.h5_micro_write(str(path), pix, rod, (12, 12, 12))
    buf = bytearray(path.read_bytes())
    name, oh, length = next(h for h in _object_headers(buf) if h[0] == "pix")
    t, at, sz = next(m for m in _messages(buf, oh, length) if m[0] == 0x000C)
    moved = bytes(buf[at: at + 8 + sz])
    eof = len(buf)
    # in place of the attribute: a continuation message and a NIL message filling the rest
    cont = struct.pack("<HHB3xQQ", 0x0010, 16, 0, eof, len(moved))
    nil = struct.pack("<HHB3x", 0x0000, sz - 16 - 8, 0) + bytes(sz - 16 - 8)
    assert len(cont) + len(nil) == 8 + sz
    buf[at: at + 8 + sz] = cont + nil
    buf += moved
    struct.pack_into("<Q", buf, 40, len(buf))
    path.write_bytes(bytes(buf))
    assert e3d.h5_micro_info(str(path))[2] == (12, 12, 12)  # the attribute, read through the continuation
    q, r = e3d.h5_micro_read(str(path), p.ns, p.nphase - 1)
    assert np.array_equal(q, pix) and np.array_equal(r, rod)


def test_big_endian_integers_are_converted(tmp_path):
    p, pix, rod = W.c2(n=8)
    path = tmp_path / "be.h5"
    e3d.h5_micro_write(str(path), pix, rod, (8, 8, 8))
    buf = bytearray(path.read_bytes())
    name, oh, length = next(h for h in _object_headers(buf) if h[0] == "pix")
    msgs = _messages(buf, oh, length)
    _, tat, _ = next(m for m in msgs if m[0] == 0x0003)
    buf[tat + 8 + 1] |= 0x01  # byte order: big endian
    _, lat, _ = next(m for m in msgs if m[0] == 0x0008)
    addr, size = struct.unpack_from("<QQ", buf, lat + 8 + 2)
    buf[addr: addr + size] = pix.astype(">i4").tobytes()
    path.write_bytes(bytes(buf))
    q, _ = e3d.h5_micro_read(str(path), p.ns, p.nphase - 1)
    assert np.array_equal(q, pix)


def test_unsupported_structures_are_refused(tmp_path):
    p, pix, rod = W.c2(n=8)
    path = tmp_path / "u.h5"
    e3d.h5_micro_write(str(path), pix, rod, (8, 8, 8))
    good = path.read_bytes()
    buf = bytearray(good)
    name, oh, length = next(h for h in _object_headers(buf) if h[0] == "pix")
    _, lat, _ = next(m for m in _messages(buf, oh, length) if m[0] == 0x0008)
    buf[lat + 8 + 1] = 2  # layout class 2: chunked
    path.write_bytes(bytes(buf))
    with pytest.raises(ValueError, match="chunked"):
        e3d.h5_micro_read(str(path), p.ns, p.nphase - 1)
    buf = bytearray(good)
    buf[8] = 2  # superblock version 2
    path.write_bytes(bytes(buf))
    with pytest.raises(ValueError, match="superblock version 2"):
        e3d.h5_micro_read(str(path), p.ns, p.nphase - 1)
    path.write_bytes(good[:200])  # truncated
    with pytest.raises(ValueError):
        e3d.h5_micro_read(str(path), p.ns, p.nphase - 1)


def test_driver_reads_hdf5_input(tmp_path):
    drv = os.path.join(os.path.dirname(e3d.LIB_PATH), "e3d_run")
    if not os.path.exists(drv):
        pytest.skip("driver not built")
    out = __import__("subprocess").run([drv, "--help"], capture_output=True, text=True)
    assert out.returncode == 0 and "--grid" in out.stdout and "fullfield_poly.h5" in out.stdout
