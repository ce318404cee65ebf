"""HDF5 files of the reference without libhdf5: the library's C++ reader and
writer (ns_h5_*, host-only, no GPU) against the oracle's NumPy reader and
writer, and both readers against a file written by the HDF5 library itself.

The reference writes snapshots with root attributes nx, dt, nu, time_scheme,
time_step, time and datasets u, v, w, p, rhs_?_previous
(big_periodic_3D.f90:630-651), sub-block records in groups "t_%.4f"
(:664-712), and restarts from snapshots (:296-324)."""
import os

import numpy as np
import pytest

from oracle import ns_h5 as H

SCIPY_H5 = None
try:
    import scipy
    _p = os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data", "testhdf5_7.4_GLNX86.mat")
    SCIPY_H5 = _p if os.path.exists(_p) else None
except ImportError:
    pass
need_libhdf5_file = pytest.mark.skipif(SCIPY_H5 is None, reason="SciPy's HDF5 test file is not installed")


def h5():
    from ns_3d_staggered_dp_gb300 import H5File
    return H5File


def ref_shapes(nx, ny, nz):
    return {"u": (nx + 1, ny + 2, nz + 2), "v": (nx + 2, ny + 1, nz + 2), "w": (nx + 2, ny + 2, nz + 1),
            "p": (nx + 2, ny + 2, nz + 2)}


# ---------------------------------------------------------------------------
# pins on a file of the HDF5 library
# ---------------------------------------------------------------------------
@need_libhdf5_file
def test_oracle_reader_on_a_libhdf5_file():
    """MATLAB's HDF5 library wrote a 1x9 double vector 0:pi/4:2*pi with the
    attribute MATLAB_class = "double", after a 512-byte user block."""
    g = H.read(SCIPY_H5)
    d = g.members["testdouble"]
    assert d.shape == (9, 1) and d.dtype == np.dtype("<f8")
    np.testing.assert_array_equal(d.data.ravel(), np.arange(9) * (np.pi / 4))
    assert d.attrs["MATLAB_class"] == "double"


@need_libhdf5_file
def test_library_reader_on_a_libhdf5_file():
    """The same file through ns_h5_open / ns_h5_read_double (Fortran shape
    (1, 9): the file's dims reversed) and a fixed string without terminator."""
    with h5()(SCIPY_H5, "r") as f:
        assert f.members("/") == ["testdouble"]
        assert f.shape("testdouble") == (1, 9)
        a = f.read("testdouble")
        np.testing.assert_array_equal(a.ravel(), np.arange(9) * (np.pi / 4))
        assert f.attr("testdouble", "MATLAB_class", str) == "double"


@need_libhdf5_file
def test_written_superblock_follows_the_library_defaults(tmp_path):
    """Version 0 superblock, 8-byte offsets and lengths, group K 4 and 16,
    as in the library's own file."""
    p = tmp_path / "a.h5"
    with h5()(p, "w") as f:
        f.write("x", np.ones(3))
    ours = open(p, "rb").read()
    theirs = open(SCIPY_H5, "rb").read()[512:]
    assert ours[:8] == theirs[:8] == H.SIG
    assert ours[8:20] == theirs[8:20]  # versions, sizes, K values


# ---------------------------------------------------------------------------
# library writer -> oracle reader
# ---------------------------------------------------------------------------
def test_snapshot_layout_reads_back_in_the_oracle(tmp_path):
    """A file laid out like the reference's snapshot: attributes typed as the
    H5LT calls type them, datasets with the Fortran dims reversed and the
    bytes of the Fortran arrays."""
    rng = np.random.default_rng(3)
    sh = ref_shapes(8, 6, 10)
    fields = {k: np.asfortranarray(rng.standard_normal(s)) for k, s in sh.items()}
    fields.update({f"rhs_{c}_previous": np.asfortranarray(rng.standard_normal(sh[k]))
                   for c, k in zip("xyz", "uvw")})
    p = tmp_path / "HIT_8^3_decay_4.E-3_AB2-CN_p_t_1.0000.h5"
    with h5()(p, "w") as f:
        f.set_attr("/", "nx", 8)
        f.set_attr("/", "dt", 4e-3)
        f.set_attr("/", "nu", 1 / 1600)
        f.set_attr("/", "time_scheme", "AB2-CN")
        f.set_attr("/", "time_step", 250)
        f.set_attr("/", "time", 1.0)
        for k, a in fields.items():
            f.write(k, a)
    g = H.read(str(p))
    assert g.attrs["nx"].dtype == np.dtype("<i4") and g.attrs["nx"].shape == (1,) and g.attrs["nx"][0] == 8
    assert g.attrs["dt"].dtype == np.dtype("<f8") and g.attrs["dt"][0] == 4e-3
    assert g.attrs["time_scheme"] == "AB2-CN" and g.attrs["time_step"][0] == 250 and g.attrs["time"][0] == 1.0
    assert sorted(g.members) == sorted(fields)
    for k, a in fields.items():
        d = g.members[k]
        assert d.shape == a.shape[::-1]
        assert d.data.tobytes() == a.tobytes(order="F")  # bit for bit


def test_record_groups_with_many_members(tmp_path):
    """300 groups t_%.4f of 30 datasets each (the sub-block records of
    :664-712 carry up to 30): a B-tree of two levels under the root and
    several symbol table nodes under every group."""
    rng = np.random.default_rng(5)
    want = {}
    p = tmp_path / "sub.h5"
    with h5()(p, "w") as f:
        f.set_attr("/", "x0", 4)
        for t in range(300):
            g = f"t_{t * 0.004:.4f}"
            f.group(g)
            for q in range(30):
                a = rng.standard_normal((2, 3) if q % 2 else (3,))
                f.write(f"{g}/d{q:02d}", a)
                want[(g, f"d{q:02d}")] = a
    g = H.read(str(p))
    assert len(g.members) == 300
    for (grp, name), a in want.items():
        np.testing.assert_array_equal(g.members[grp].members[name].data, np.asarray(a).T)
    with h5()(p, "r") as f:
        assert len(f.members("/")) == 300
        np.testing.assert_array_equal(f.read("t_0.4000/d07"), want[("t_0.4000", "d07")])


def test_flush_leaves_a_complete_file(tmp_path):
    """Every flush writes a readable file (the reference closes and reopens
    its record files for this); later writes add to it."""
    p = tmp_path / "f.h5"
    f = h5()(p, "w")
    f.write("a", np.arange(4.0))
    f.flush()
    assert list(H.read(str(p)).members) == ["a"]
    f.group("g")
    f.write("g/b", np.ones((2, 2)))
    f.close()
    g = H.read(str(p))
    assert sorted(g.members) == ["a", "g"] and g.members["g"].members["b"].shape == (2, 2)


# ---------------------------------------------------------------------------
# oracle writer -> library reader, and appending to it
# ---------------------------------------------------------------------------
def _grown_file():
    rng = np.random.default_rng(9)
    root = H.Group(attrs={"nx": 16, "dt": 2.5e-4, "time_scheme": "AB2"})
    for t in range(45):
        grp = H.Group(attrs={"k": t})
        for q in range(11):
            d = rng.standard_normal((3, 2, 4)) if q else rng.standard_normal((2,))  # the short one is compact
            grp.members[f"f{q:02d}"] = H.Dataset(d.shape, np.dtype("<f8"), d)
        root.members[f"t_{t:.4f}"] = grp
    return root


def test_library_reader_on_a_grown_file(tmp_path):
    """A user block, object headers split by continuations, half-full
    symbol table and B-tree nodes over three levels, version 2 contiguous
    and version 3 compact layouts."""
    root = _grown_file()
    p = tmp_path / "grown.h5"
    p.write_bytes(H.write(root, userblock=512, leaf_fill=4, node_fill=4))
    with h5()(p, "r") as f:
        assert f.members("/") == [k + "/" for k in sorted(root.members)]  # groups end in "/"
        assert f.attr("/", "time_scheme", str) == "AB2" and f.attr("/", "nx", int) == 16
        assert f.attr("/", "dt") == 2.5e-4
        for k, grp in root.members.items():
            assert f.attr(k, "k", int) == grp.attrs["k"]
            for q, d in grp.members.items():
                np.testing.assert_array_equal(f.read(f"{k}/{q}"), d.data.T)


def test_append_keeps_what_the_file_holds(tmp_path):
    """h5fopen_f with H5F_ACC_RDWR_F: new groups, datasets and attributes are
    added; the old ones (user block included) read back unchanged."""
    root = _grown_file()
    p = tmp_path / "grown.h5"
    p.write_bytes(H.write(root, userblock=512, leaf_fill=4, node_fill=4))
    with h5()(p, "a") as f:
        f.group("t_99.0000")
        f.write("t_99.0000/u_sub", np.arange(12.0).reshape(3, 4))
        f.set_attr("/", "time", 3.5)
        f.set_attr("/", "nx", 32)  # replaced, not duplicated
    g = H.read(str(p))
    assert g.attrs["time"][0] == 3.5 and g.attrs["nx"][0] == 32 and g.attrs["time_scheme"] == "AB2"
    np.testing.assert_array_equal(g.members["t_99.0000"].members["u_sub"].data, np.arange(12.0).reshape(3, 4).T)
    for k, grp in root.members.items():
        for q, d in grp.members.items():
            np.testing.assert_array_equal(g.members[k].members[q].data, d.data)


# ---------------------------------------------------------------------------
# errors
# ---------------------------------------------------------------------------
def test_errors_are_statuses(tmp_path):
    from ns_3d_staggered_dp_gb300 import NSError
    F = h5()
    p = tmp_path / "e.h5"
    with F(p, "w") as f:
        f.write("a", np.zeros((2, 3)))
        with pytest.raises(NSError) as e:
            f.write("a", np.zeros(2))            # exists
        assert e.value.status == 6
        with pytest.raises(NSError) as e:
            f.write("nogroup/a", np.zeros(2))    # parent missing (h5gcreate_f first)
        assert e.value.status == 6
    with pytest.raises(NSError) as e:
        F(p, "w")                                # H5F_ACC_EXCL_F
    assert e.value.status == 8
    with F(p, "r") as f:
        with pytest.raises(NSError) as e:
            f.read("a", (3, 2))                  # the buffer's dims differ
        assert e.value.status == 1
        with pytest.raises(NSError) as e:
            f.read("b", (2, 3))
        assert e.value.status == 6
        with pytest.raises(NSError) as e:
            f.group("g")                         # read-only
        assert e.value.status == 6
    (tmp_path / "not.h5").write_bytes(b"not an hdf5 file" * 64)
    with pytest.raises(NSError) as e:
        F(tmp_path / "not.h5", "r")
    assert e.value.status == 8
    good = p.read_bytes()
    (tmp_path / "cut.h5").write_bytes(good[: len(good) // 2])
    with pytest.raises(NSError) as e:
        F(tmp_path / "cut.h5", "r")              # truncated
    assert e.value.status == 8


def test_outside_the_subset_is_refused(tmp_path):
    """A version 2 object header (the library's newer format) is reported
    as NS_ERR_IO, not misread."""
    from ns_3d_staggered_dp_gb300 import NSError
    b = bytearray(H.write(H.Group(members={"a": H.Dataset((4,), np.dtype("<f8"), np.arange(4.0))}),
                          userblock=0, split_headers=False))
    g = H._Reader(bytes(b))
    _n, oh, _c = g.entry_abs(g.root_entry)
    b[oh] = 2  # root object header version
    (tmp_path / "v2.h5").write_bytes(bytes(b))
    with pytest.raises(NSError) as e:
        h5()(tmp_path / "v2.h5", "r")
    assert e.value.status == 8
