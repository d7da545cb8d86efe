"""The HDF5 field output (src/hdf5_io.F90, src/WriteOutput_corner1.F90:21-78)
written without libhdf5.

The reader is pinned to a file libhdf5 itself wrote (the HDF5-format MAT file
that scipy ships among its test data: user block, superblock version 0,
symbol-table root group, one 1x9 FP64 dataset with a string attribute).  The
writer is then checked through that reader (the reference's own
write-then-read unit tests, test/test_hdf5_io.f90, with their inputs) and
against the structural invariants of the format on the bytes themselves."""
import struct
from pathlib import Path

import numpy as np
import pytest

from biocfd import h5io


def _libhdf5_file():
    scipy_io = pytest.importorskip("scipy.io.matlab")
    p = Path(scipy_io.__file__).parent / "tests" / "data" / "testhdf5_7.4_GLNX86.mat"
    if not p.exists():
        pytest.skip("scipy's HDF5 test file is not installed")
    return p


def test_reader_reads_a_file_written_by_libhdf5():
    root = h5io.read_file(_libhdf5_file())
    assert list(root.children) == ["testdouble"]
    d = root.children["testdouble"]
    assert d.dims == (9, 1) and d.dtype == np.dtype("<f8")
    np.testing.assert_allclose(d.read().ravel(), np.arange(9) * np.pi / 4, rtol=0, atol=1e-15)
    assert d.attrs == {"MATLAB_class": b"double"}


# test/test_hdf5_io.f90: every case writes to the same file and group
GROUP = "/test_group"


def _ref_arrays():
    i, j, k = np.meshgrid(np.arange(1, 5), np.arange(1, 4), np.arange(1, 3), indexing="ij")
    a3 = np.asfortranarray(i + 10 * j + 100 * k)
    j2, k2 = np.meshgrid(np.arange(1, 4), np.arange(1, 3), indexing="ij")
    a2 = np.asfortranarray(10 * j2 + 100 * k2)
    a1 = 100 * np.arange(1, 3)
    return a3, a2, a1


def test_reference_unit_cases_round_trip(tmp_path):
    fn = str(tmp_path / "test_output.h5")
    a3, a2, a1 = _ref_arrays()
    h5io.hdf5_write_real(fn, array_input_3d=a3.astype(float), key="3d_real_array", group=GROUP)
    h5io.hdf5_write_real(fn, array_input_2d=a2.astype(float), key="2d_real_array", group=GROUP)
    h5io.hdf5_write_real(fn, array_input_1d=a1.astype(float), key="1d_real_array", group=GROUP)
    h5io.hdf5_write_real(fn, scalar_input=20.5, key="real_scalar", group=GROUP)
    h5io.hdf5_write_int(fn, array_input_3d=a3, key="3d_integer_array", group=GROUP)
    h5io.hdf5_write_int(fn, array_input_2d=a2, key="2d_integer_array", group=GROUP)
    h5io.hdf5_write_int(fn, array_input_1d=a1, key="1d_integer_array", group=GROUP)
    h5io.hdf5_write_int(fn, scalar_input=20, key="integer_scalar", group=GROUP)

    r3 = h5io.hdf5_read_real_3d(fn, GROUP, "3d_real_array")
    assert r3.shape == (4, 3, 2) and r3.dtype == np.float64 and np.array_equal(r3, a3)
    assert np.array_equal(h5io.hdf5_read_real_2d(fn, GROUP, "2d_real_array"), a2)
    assert np.array_equal(h5io.hdf5_read_real_1d(fn, GROUP, "1d_real_array"), a1)
    assert h5io.hdf5_read_real_scalar(fn, GROUP, "real_scalar") == 20.5
    i3 = h5io.hdf5_read_int_3d(fn, GROUP, "3d_integer_array")
    assert i3.dtype == np.int64 and np.array_equal(i3, a3)
    assert np.array_equal(h5io.hdf5_read_int_2d(fn, GROUP, "2d_integer_array"), a2)
    assert np.array_equal(h5io.hdf5_read_int_1d(fn, GROUP, "1d_integer_array"), a1)
    assert h5io.hdf5_read_int_scalar(fn, GROUP, "integer_scalar") == 20

    # the Fortran API's layout: file dims reversed, raw data in Fortran order
    d = h5io.read_file(fn).find(GROUP).children["3d_real_array"]
    assert d.dims == (2, 3, 4)
    raw = np.fromfile(fn, dtype="<f8", count=24, offset=d.addr)
    assert np.array_equal(raw, a3.ravel(order="F"))


def test_one_input_per_call(tmp_path):
    fn = str(tmp_path / "x.h5")
    with pytest.raises(ValueError, match="More than one argument"):
        h5io.hdf5_write_real(fn, scalar_input=1.0, array_input_1d=np.zeros(2), key="a", group="/")
    with pytest.raises(TypeError):
        h5io.hdf5_write_int(fn, array_input_1d=np.zeros(2), key="a", group="/")
    with pytest.raises(ValueError):
        h5io.hdf5_write_real(fn, array_input_3d=np.zeros((2, 2)), key="a", group="/")


def _u64(b, off):
    return struct.unpack_from("<Q", b, off)[0]


def _structure(fn):
    """Checks the format's invariants on the raw bytes, independently of
    the reader; returns the root group's (B-tree children, names)."""
    b = Path(fn).read_bytes()
    assert b[:8] == h5io.SIGNATURE
    assert b[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])            # versions, 8-byte offsets/lengths
    assert struct.unpack_from("<HHI", b, 16) == (4, 16, 0)     # leaf K, internal K, flags
    assert _u64(b, 24) == 0 and _u64(b, 32) == h5io.UNDEF      # base, free space
    assert _u64(b, 40) == len(b) and _u64(b, 48) == h5io.UNDEF  # end of file, driver
    name_off, oh, cache = _u64(b, 56), _u64(b, 64), struct.unpack_from("<I", b, 72)[0]
    bt, hp = _u64(b, 80), _u64(b, 88)
    assert name_off == 0 and cache == 1
    # root object header: version 1, messages fill the chunk, symbol table matches the cache
    ver, nmsg, size = b[oh], struct.unpack_from("<H", b, oh + 2)[0], struct.unpack_from("<I", b, oh + 8)[0]
    assert ver == 1 and oh % 8 == 0
    p, seen = oh + 16, []
    while p < oh + 16 + size:
        t, sz = struct.unpack_from("<HH", b, p)
        assert sz % 8 == 0
        seen.append(t)
        if t == h5io.MSG_STAB:
            assert (_u64(b, p + 8), _u64(b, p + 16)) == (bt, hp)
        p += 8 + sz
    assert p == oh + 16 + size and len(seen) == nmsg and seen[0] == h5io.MSG_STAB
    # heap: empty name at offset 0, data segment right after the 32-byte prefix
    assert b[hp:hp + 4] == b"HEAP" and _u64(b, hp + 24) == hp + 32 and _u64(b, hp + 16) == 1
    seg = b[hp + 32:hp + 32 + _u64(b, hp + 8)]
    assert seg[:8] == bytes(8)
    name = lambda o: seg[o:seg.index(b"\0", o)]
    # B-tree: one leaf-level node, keys bracket each symbol-table node's names
    assert b[bt:bt + 4] == b"TREE" and b[bt + 4] == 0 and b[bt + 5] == 0
    n = struct.unpack_from("<H", b, bt + 6)[0]
    vals = struct.unpack_from(f"<{2 * n + 1}Q", b, bt + 24)
    names = []
    for i in range(n):
        sn = vals[2 * i + 1]
        assert b[sn:sn + 4] == b"SNOD" and b[sn + 4] == 1
        m = struct.unpack_from("<H", b, sn + 6)[0]
        assert 1 <= m <= 8
        nm = [name(_u64(b, sn + 8 + 40 * j)) for j in range(m)]
        assert nm == sorted(nm) and name(vals[2 * i]) < nm[0] and nm[-1] == name(vals[2 * i + 2])
        names += nm
    assert names == sorted(names) and len(set(names)) == len(names)
    return n, [x.decode() for x in names]


def test_field_file_of_write_output_hdf5(tmp_path):
    rng = np.random.default_rng(7)
    nx, ny, nz = 5, 4, 3
    shp = (nx + 2, ny + 2, nz + 2)
    f = {k: np.asfortranarray(rng.standard_normal(shp)) for k in ("u", "v", "w", "p")}
    tags = {k: np.asfortranarray(rng.integers(-3, 4, shp).astype(np.int32)) for k in ("cell", "cell_n", "cell_pr")}
    x1, y1, z1 = (np.cumsum(rng.uniform(0.5, 1.0, m + 3)) for m in (nx, ny, nz))
    path = tmp_path / h5io.field_name_hdf5(400, 2)
    assert str(path).endswith("out/timestep_00400_block_00002.h5")
    h5io.write_fields_hdf5(path, x1, y1, z1, f, tags, 0.125)

    nsnod, names = _structure(path)
    assert nsnod == 2  # ten datasets: more than one symbol-table node's eight entries
    assert names == sorted(["u1", "v1", "w1", "xp", "yp", "zp", "p", "cell", "cell_n", "cell_pr"])
    r = lambda k: h5io.hdf5_read_real_3d(path, "/", k)
    i = (slice(1, -1),) * 3
    assert np.array_equal(r("u1"), 0.5 * (f["u"][i] + f["u"][:-2, 1:-1, 1:-1]))
    assert np.array_equal(r("v1"), 0.5 * (f["v"][i] + f["v"][1:-1, :-2, 1:-1]))
    assert np.array_equal(r("w1"), 0.5 * (f["w"][i] + f["w"][1:-1, 1:-1, :-2]))
    assert np.array_equal(r("p"), f["p"][i])
    assert np.array_equal(h5io.hdf5_read_real_1d(path, "/", "xp"), 0.5 * (x1[1:] + x1[:-1])[1:nx + 1])
    assert np.array_equal(h5io.hdf5_read_real_1d(path, "/", "zp"), 0.5 * (z1[1:] + z1[:-1])[1:nz + 1])
    for k in ("cell", "cell_n", "cell_pr"):
        assert np.array_equal(h5io.hdf5_read_int_3d(path, "/", k), tags[k][i])
    # zonej carries nx, as the reference writes it
    assert [h5io.hdf5_read_int_scalar(path, "/", k) for k in ("zonei", "zonej", "zonek")] == [nx, nx, nz]
    assert h5io.hdf5_read_real_scalar(path, "/", "totime") == 0.125


def test_groups_many_names_and_replacement(tmp_path):
    fn = tmp_path / "g.h5"
    keys = [f"k{q:02d}" for q in range(40)] + ["A", "Z", "_"]
    for q, k in enumerate(keys):
        h5io.hdf5_write_real(fn, array_input_1d=np.arange(q + 1, dtype=float), key=k, group="/a/b")
    h5io.hdf5_write_int(fn, scalar_input=3, key="n", group="/a")
    h5io.hdf5_write_real(fn, array_input_1d=np.full(3, 7.0), key="k05", group="/a/b")
    root = h5io.read_file(fn)
    b = root.find("/a/b")
    assert list(b.children) == sorted(keys, key=str.encode)
    for q, k in enumerate(keys):
        want = np.full(3, 7.0) if k == "k05" else np.arange(q + 1, dtype=float)
        assert np.array_equal(h5io.hdf5_read_real_1d(fn, "/a/b", k), want)
    assert root.find("a").attrs == {"n": 3}
    _structure(fn)


def test_rejects_what_is_not_hdf5(tmp_path):
    p = tmp_path / "bad.h5"
    p.write_bytes(b"not an hdf5 file" * 40)
    with pytest.raises(h5io.H5FormatError):
        h5io.read_file(p)
    good = tmp_path / "good.h5"
    h5io.hdf5_write_real(good, array_input_1d=np.ones(4), key="x", group="/")
    b = bytearray(good.read_bytes())
    oh = _u64(b, 64)
    b[oh + 2] += 1  # message count no longer matches the messages
    p.write_bytes(bytes(b))
    with pytest.raises(h5io.H5FormatError, match="messages"):
        h5io.read_file(p)


def test_truncated_file_is_a_format_error(tmp_path):
    good = tmp_path / "good.h5"
    h5io.hdf5_write_real(good, array_input_1d=np.ones(4), key="x", group="/")
    b = good.read_bytes()
    bad = tmp_path / "cut.h5"
    for cut in (100, len(b) // 2, len(b) - 8):
        bad.write_bytes(b[:cut])
        with pytest.raises(h5io.H5FormatError):
            h5io.read_file(bad).children["x"].read()
