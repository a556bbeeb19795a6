"""The library's HDF5 writer (tdz_h5_write, tdz_obsfile_*; host code, no
GPU): files in the classic layout the HDF5 library itself writes, read back
by the strict reader tests/h5lite.py.

The reader is pinned on a file that the HDF5 library wrote (the MATLAB 7.3
test file that scipy ships, an HDF5 file behind a 512-byte user block): it
reads the array scipy's own reader gets from the MATLAB 5 twin of that file.
The writer's superblock fields and its fill-value, datatype, dataspace and
layout messages are compared byte for byte with that file's; then the
observables file of the reference's schema (src/manager.cpp:51-201) and flat
files with attributes (src/tsurff.cpp:1018-1057) are read back exactly."""
import ctypes as C
import os
import struct

import numpy as np
import pytest

from tests import h5lite

MATLAB_DATA = None
try:
    import scipy.io.matlab as _sm
    MATLAB_DATA = os.path.join(os.path.dirname(_sm.__file__), "tests", "data")
except Exception:
    pass
LIB_FILE = os.path.join(MATLAB_DATA or "", "testhdf5_7.4_GLNX86.mat")
V5_TWIN = os.path.join(MATLAB_DATA or "", "testdouble_7.4_GLNX86.mat")


@pytest.fixture(scope="module")
def lib():
    from tdsez_gb300 import _lib, build
    build.build()
    return _lib.load()


def library_file():
    if not os.path.exists(LIB_FILE):
        pytest.skip("no HDF5 file written by the HDF5 library on this host")
    return h5lite.File(LIB_FILE)


def test_reader_pins_on_a_library_written_file():
    f = library_file()
    assert f.base == 512 and f.superblock["version"] == 0
    assert f.keys() == ["testdouble"]
    d = f["testdouble"]
    assert d.shape == (9, 1) and d.dtype == np.dtype("<f8")
    assert bytes(d.attrs["MATLAB_class"]) == b"double"
    import scipy.io as sio
    twin = sio.loadmat(V5_TWIN)["testdouble"]
    assert np.array_equal(d.read().T, twin)
    assert np.array_equal(d.read().ravel(), np.arange(9) * np.pi / 4)


def _msgs_by_type(msgs):
    out = {}
    for t, fl, body in msgs:
        out.setdefault(t, []).append((fl, body))
    return out


def test_writer_uses_the_library_encodings(lib, tmp_path):
    from tdsez_gb300.outputs import write_h5
    ref = library_file()
    vals = np.arange(9, dtype=np.float64).reshape(9, 1) * np.pi / 4
    path = tmp_path / "one.h5"
    write_h5(path, {"testdouble": vals})
    raw = path.read_bytes()
    ours = h5lite.File(str(path))
    ref_raw = open(LIB_FILE, "rb").read()[512:]
    # superblock: versions, offset/length sizes, group K values
    assert raw[:8] == ref_raw[:8] == h5lite.SIGNATURE
    assert raw[8:20] == ref_raw[8:20]
    assert struct.unpack_from("<Q", raw, 40)[0] == len(raw)
    # root symbol-table entry: a group (cache type 1) with its B-tree and heap
    assert ours.superblock["root"]["cache"] == ref.superblock["root"]["cache"] == 1
    assert np.array_equal(ours["testdouble"].read(), vals)
    a, b = _msgs_by_type(ours["testdouble"].messages), _msgs_by_type(ref["testdouble"].messages)
    for t in (0x5, 0x3, 0x1):   # fill value, datatype, dataspace: identical bytes and flags
        assert a[t] == b[t], hex(t)
    (fa, la), (fb, lb) = a[0x8][0], b[0x8][0]   # layout: identical but for the data address
    assert fa == fb and la[:8] == lb[:8] and la[16:] == lb[16:]
    ra, rb = _msgs_by_type(ours.messages), _msgs_by_type(ref.messages)
    assert [fl for fl, _ in ra[0x11]] == [fl for fl, _ in rb[0x11]]


def test_observables_file_round_trip(lib, tmp_path):
    from tdsez_gb300.outputs import SETS, ObservablesFile
    rng = np.random.default_rng(5)
    for dim, nb in ((1, 0), (2, 3), (3, 1)):
        path = tmp_path / f"obs{dim}.h5"
        f = ObservablesFile(path, dim, nb, flush_rows=4)
        assert f.columns == {"dipoles": 1 + 3 * dim, "populations": 1 + nb, "energies": 7,
                             "currents": 15 if dim == 3 else 11, "autocorrelation": 3}
        expect = {s: [] for s in SETS}
        for r in range(10):
            t = 0.05 * r
            row = {}
            for s in SETS:
                if (r + len(s)) % 3 == 0:
                    continue          # not supplied: zeros
                row[s] = rng.standard_normal(f.columns[s] - 1)
            f.record(t, **row)
            for s in SETS:
                expect[s].append(np.concatenate([[t], row.get(s, np.zeros(f.columns[s] - 1))]))
            if r == 2:
                assert f.rows == (3, 0) and not path.exists()
            if r == 3:
                assert f.rows == (4, 4)
                assert h5lite.File(str(path))["dipoles"].shape == (4, 1 + 3 * dim)
        assert f.rows == (10, 8)
        f.close()
        h = h5lite.File(str(path))
        assert h.keys() == sorted(SETS)
        for s in SETS:
            got = h[s].read()
            assert got.dtype == np.float64 and np.array_equal(got, np.array(expect[s])), s
        with pytest.raises(ValueError):
            f.record(0.0)


def test_observables_rows_are_checked(lib, tmp_path):
    from tdsez_gb300.outputs import ObservablesFile
    with ObservablesFile(tmp_path / "o.h5", 2) as f:
        with pytest.raises(ValueError):
            f.record(0.0, dipoles=np.zeros(7))       # 6 values after the time in 2D
        with pytest.raises(ValueError):
            f.record(0.0, energy=np.zeros(6))
        f.record(0.0, energies=np.arange(6.0))
    h = h5lite.File(str(tmp_path / "o.h5"))
    assert np.array_equal(h["energies"].read(), [[0.0, 0, 1, 2, 3, 4, 5]])
    assert np.array_equal(h["populations"].read(), [[0.0]])


def test_flat_file_with_attributes(lib, tmp_path):
    from tdsez_gb300.outputs import write_h5
    rng = np.random.default_rng(11)
    ds = {f"set_{i:02d}": rng.standard_normal([(3, ), (4, 5), (2, 3, 4)][i % 3]) for i in range(12)}
    ds["B_upper"] = rng.standard_normal(7)      # byte order: upper case sorts first
    ds["pes_grid"] = rng.standard_normal((6, 5, 4))
    attrs = {"final_time": 16.0, "radius": 10.0, "A_final": [0.1, -0.2, 0.3], "n_samples": 641.0}
    path = tmp_path / "sub" / "surff.h5"
    write_h5(path, ds, attrs)
    f = h5lite.File(str(path))
    assert f.keys() == sorted(ds, key=lambda s: s.encode())
    assert f.leaf_k == 7           # 14 names: symbol-table nodes of 2 K = 14 entries
    for k, v in ds.items():
        assert np.array_equal(f[k].read(), v), k
    assert set(f.attrs) == set(attrs)
    for k, v in attrs.items():
        assert np.array_equal(f.attrs[k], np.atleast_1d(v)), k
    assert not os.path.exists(str(path) + ".part")


def test_writer_rejects_bad_input(lib, tmp_path):
    from tdsez_gb300 import _lib
    from tdsez_gb300.outputs import write_h5
    bad = [({"a": np.zeros(2), "b/c": np.zeros(2)}, "invalid dataset name"),
           ({".": np.zeros(2)}, "invalid dataset name"),
           ({"a": np.zeros((0, 3))}, "empty axis")]
    for ds, msg in bad:
        with pytest.raises(_lib.TDZError) as e:
            write_h5(tmp_path / "bad.h5", ds)
        assert e.value.status == 1 and msg in str(e.value)
    with pytest.raises(_lib.TDZError):
        write_h5(tmp_path / "bad.h5", {"a": np.zeros(2)}, {"a": 1.0, "a ": 2.0, "x/y": 3.0})
    assert not (tmp_path / "bad.h5").exists()
    st = lib.tdz_obsfile_open(str(tmp_path / "x.h5").encode(), 4, 0, 0, C.byref(C.c_void_p()))
    assert st == 1 and b"dimension" in lib.tdz_last_error()
