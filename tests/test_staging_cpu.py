"""Staged-input cache (HDF5): the format layer and the reference's file layout.

* ``staged_<case>.h5`` were written by the reference's own ``dump``
  (trot/staging.py:843-854, 1353-1375; tests/golden/make_staged_golden.py):
  ``trot_gb300.staging.load`` must return the inputs recorded beside them, and
  ``trot_gb300.staging.dump`` of those inputs must write the same bytes.
* An HDF5 file written by another implementation (MATLAB's HDF5 library; it ships
  with scipy's test data) is read and compared with scipy's reading of the same
  variable from the MATLAB-format copy.
"""
from __future__ import annotations

import json
import os
import struct
import zlib

import numpy as np
import pytest

from trot_gb300 import h5file, staging

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["rhf", "uhf", "cisd"]


def _inputs(case):
    z = np.load(os.path.join(GOLDEN, f"staged_{case}.npz"))
    ham = {k[4:]: z[k] for k in z.files if k.startswith("ham.")}
    trial = {k[6:]: z[k] for k in z.files if k.startswith("trial.")}
    data = {k[5:]: z[k] for k in z.files if k.startswith("data.")}
    meta = json.loads(str(z["meta_json"]))
    frozen = lambda v: v if v.ndim else int(v)  # noqa: E731
    h = staging.HamInput(h0=float(ham["h0"]), h1=ham["h1"], chol=ham["chol"], nelec=tuple(int(x) for x in ham["nelec"]),
                         norb=int(ham["norb"]), chol_cut=float(ham["chol_cut"]), frozen=frozen(ham["frozen"]),
                         source_kind=str(ham["source_kind"]), basis=str(ham["basis"]))
    t = staging.TrialInput(kind=str(trial["kind"]), data=data, frozen=frozen(trial["frozen"]),
                           source_kind=str(trial["source_kind"]))
    return staging.StagedInputs(ham=h, trial=t, meta=meta)


def _eq(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a, b)


@pytest.mark.parametrize("case", CASES)
def test_load_reference_dump(case):
    want = _inputs(case)
    got = staging.load(os.path.join(GOLDEN, f"staged_{case}.h5"))
    for f in ("h0", "nelec", "norb", "chol_cut", "source_kind", "basis"):
        assert getattr(got.ham, f) == getattr(want.ham, f), f
    assert _eq(got.ham.h1, want.ham.h1) and _eq(got.ham.chol, want.ham.chol)
    assert _eq(got.ham.frozen, want.ham.frozen) and type(got.ham.frozen) is type(want.ham.frozen)
    assert got.trial.kind == want.trial.kind and got.trial.source_kind == want.trial.source_kind
    assert _eq(got.trial.frozen, want.trial.frozen)
    assert sorted(got.trial.data) == sorted(want.trial.data)
    for k, v in want.trial.data.items():
        assert _eq(got.trial.data[k], v), k
    meta = dict(want.meta)
    meta["frozen"] = staging._freeze_from_meta_value(meta["frozen"])
    assert json.dumps(got.meta, default=lambda a: a.tolist()) == json.dumps(meta, default=lambda a: a.tolist())


@pytest.mark.parametrize("case", CASES)
def test_dump_matches_reference_bytes(case, tmp_path):
    """Same inputs, same call sequence as the reference's _dump_h5: identical files."""
    p = tmp_path / "ours.h5"
    staging.dump(_inputs(case), p)
    with open(os.path.join(GOLDEN, f"staged_{case}.h5"), "rb") as f:
        assert p.read_bytes() == f.read()


def test_matlab_hdf5_file():
    sio = pytest.importorskip("scipy.io")
    import scipy.io.matlab as sm
    data = os.path.join(os.path.dirname(sm.__file__), "tests", "data")
    h5 = os.path.join(data, "testhdf5_7.4_GLNX86.mat")
    v5 = os.path.join(data, "testdouble_7.4_GLNX86.mat")
    if not (os.path.exists(h5) and os.path.exists(v5)):
        pytest.skip("scipy's MATLAB test files are not installed")
    with h5file.File(h5) as f:  # 512-byte user block before the superblock
        assert f.keys() == ["testdouble"]
        ds = f["testdouble"]
        assert ds.attrs["MATLAB_class"] == b"double"
        got = np.asarray(ds)
    want = sio.loadmat(v5)["testdouble"]
    assert got.dtype == np.float64 and np.array_equal(got, want.T)  # MATLAB stores column-major


def test_types_groups_attrs_roundtrip(tmp_path):
    rng = np.random.default_rng(3)
    arrays = {
        "f8": rng.normal(size=(4, 5, 6)), "f4": rng.normal(size=(7,)).astype(np.float32),
        "i8": rng.integers(-9, 9, size=(3, 2)), "i4": np.arange(5, dtype=np.int32), "u1": np.arange(9, dtype=np.uint8),
        "c16": rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3)), "c8": (np.arange(4) * (1 + 2j)).astype(np.complex64),
        "scalar": np.array(2.5), "empty": np.zeros((0, 3)), "bytes": np.array([b"ab", b"xyz"]),
        "big_endian": np.arange(6, dtype=">f8").reshape(2, 3),
    }
    p = tmp_path / "t.h5"
    with h5file.File(p, "w") as f:
        g = f.create_group("a/b")
        for k, v in arrays.items():
            g.create_dataset(k, data=v)
        many = f.create_group("many")  # 40 members: five symbol-table nodes under one B-tree node
        for i in range(40):
            many.create_dataset(f"m{39 - i:02d}", data=np.full(2, i))
        f.attrs["text"] = "héllo ✓"
        f.attrs["i"] = 7
        f.attrs["x"] = -1e-300
        f.attrs["vec"] = np.array([1.0, 2.0])
        g.attrs["t2"] = "second"
        g["f8"].attrs["units"] = "Ha"
    with h5file.File(p) as f:
        assert sorted(f.keys()) == ["a", "many"]
        assert f.attrs["text"] == "héllo ✓" and f.attrs["i"] == 7 and f.attrs["x"] == -1e-300
        assert isinstance(f.attrs["i"], np.int64)
        assert _eq(f.attrs["vec"], [1.0, 2.0])
        g = f["a"]["b"]
        assert g.attrs["t2"] == "second" and f["a/b/f8"].attrs["units"] == "Ha"
        for k, v in arrays.items():
            got = np.asarray(g[k])
            want = v.astype(v.dtype.newbyteorder("<")) if k == "big_endian" else v
            assert _eq(got, want), k
        assert sorted(f["many"].keys()) == [f"m{i:02d}" for i in range(40)]
        for i in range(40):
            assert _eq(f["many"][f"m{39 - i:02d}"][...], np.full(2, i))
        assert "a/b/f8" in f and "a/b/nope" not in f and "nope" not in f
        off, n = f["a/b/f8"].extent()
        assert n == arrays["f8"].nbytes and off % 64 == 0
        out = np.empty((4, 5, 6))
        f["a/b/f8"].read_into(out)
        assert _eq(out, arrays["f8"])


def test_refusals(tmp_path):
    p = tmp_path / "r.h5"
    with h5file.File(p, "w") as f:
        with pytest.raises(TypeError):
            f.create_dataset("obj", data=np.array([object()]))
        with pytest.raises(TypeError):
            f.attrs["flag"] = True
        g = f.create_group("g")
        with pytest.raises(ValueError):
            f.create_group("g")
        for i in range(2 * 16 * 8 + 1):
            g.create_dataset(f"d{i}", data=np.zeros(1))
        with pytest.raises(NotImplementedError):
            f.close()
    with pytest.raises(OSError):
        h5file.File(os.path.join(GOLDEN, "staged_rhf.npz"))
    with h5file.File(os.path.join(GOLDEN, "staged_rhf.h5")) as f:
        with pytest.raises(OSError):
            f.attrs["x"] = 1
        with pytest.raises(KeyError):
            f["missing"]


def _chunked_file(path, arr, chunk, filters):
    """A file whose dataset "x" is chunked: built with this package's writer, with the
    dataset's header swapped for a chunked layout, a filter pipeline and a version-1
    B-tree over the chunks (laid out by the format specification)."""
    w_dataset = h5file._FileWriter._dataset

    def chunked(self, ds):
        rank = arr.ndim
        grid = [range(0, s, c) for s, c in zip(arr.shape, chunk)]
        keys, addrs = [], []
        for idx in np.ndindex(*[len(g) for g in grid]):
            off = [g[i] for g, i in zip(grid, idx)]
            block = np.zeros(chunk, arr.dtype)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(off, chunk, arr.shape))
            block[tuple(slice(0, s.stop - s.start) for s in sl)] = arr[sl]
            raw = block.tobytes()
            if "shuffle" in filters:
                a = np.frombuffer(raw, np.uint8).reshape(-1, arr.itemsize)
                raw = a.T.tobytes()
            if "deflate" in filters:
                raw = zlib.compress(raw)
            self._align()
            addrs.append(self._append(raw))
            keys.append(struct.pack("<II", len(raw), 0) + struct.pack(f"<{rank + 1}Q", *off, 0))
        end = struct.pack("<II", 0, 0) + struct.pack(f"<{rank + 1}Q", *arr.shape, 0)
        tree = b"TREE" + bytes([1, 0]) + struct.pack("<HQQ", len(keys), h5file.UNDEF, h5file.UNDEF)
        for k, a in zip(keys, addrs):
            tree += k + struct.pack("<Q", a)
        tree += end
        self._align()
        bt = self._append(tree)
        layout = struct.pack("<BBB", 3, 2, rank + 1) + struct.pack("<Q", bt) + struct.pack(
            f"<{rank + 1}I", *chunk, arr.itemsize)
        pipe = b""
        names = [f for f in ("shuffle", "deflate") if f in filters]  # applied in this order on write
        for f in names:
            fid, cd = (2, [arr.itemsize]) if f == "shuffle" else (1, [6])
            pipe += struct.pack("<HHHH", fid, 0, 0, len(cd)) + struct.pack(f"<{len(cd)}I", *cd)
            pipe += b"\0" * 4 if len(cd) % 2 else b""
        msgs = [(0x01, 0, h5file._dataspace(arr.shape)), (0x03, 1, h5file._encode_dtype(arr.dtype)),
                (0x08, 0, layout)]
        if names:
            msgs.append((0x0B, 0, bytes([1, len(names)]) + b"\0" * 6 + pipe))
        return self._object_header(msgs)

    h5file._FileWriter._dataset = chunked
    try:
        with h5file.File(path, "w") as f:
            f.create_dataset("x", data=np.zeros(1))
    finally:
        h5file._FileWriter._dataset = w_dataset


@pytest.mark.parametrize("filters", [(), ("deflate",), ("shuffle", "deflate")])
def test_chunked_reader(tmp_path, filters):
    arr = np.random.default_rng(5).normal(size=(7, 10))
    p = tmp_path / "c.h5"
    _chunked_file(p, arr, (3, 4), filters)
    with h5file.File(p) as f:
        assert f["x"].extent() is None
        assert _eq(np.asarray(f["x"]), arr)


def _v2_file(path, arr, sub):
    """A file in the newer format (as libver="latest" writers lay it out): superblock
    version 2, version-2 object headers (OHDR, one continuation chunk OCHK), groups held
    as link messages, a version-3 attribute, a version-2 dataspace and a version-3
    fill-value message. Checksums are left zero (the reader does not verify them)."""
    buf = bytearray(b"\0" * 48)  # superblock, written last

    def put(b):
        while len(buf) % 8:
            buf.append(0)
        at = len(buf)
        buf.extend(b)
        return at

    def msg(t, data, flags=0):
        return struct.pack("<BHB", t, len(data), flags) + data

    def ohdr(msgs):
        body = b"".join(msgs)
        return b"OHDR" + bytes([2, 0x02]) + struct.pack("<I", len(body)) + body + b"\0" * 4  # 4-byte chunk size

    def dataset(a):
        data_at = put(a.tobytes())
        space = bytes([2, a.ndim, 0, 1]) + struct.pack(f"<{a.ndim}Q", *a.shape)
        layout = struct.pack("<BBQQ", 3, 1, data_at, a.nbytes)
        fill = bytes([3, 0x09])  # version 3: early allocation, never write fill values
        return put(ohdr([msg(0x01, space), msg(0x03, h5file._encode_dtype(a.dtype), 1), msg(0x05, fill),
                         msg(0x08, layout)]))

    def link(name, addr):
        nb = name.encode()
        return bytes([1, 0x00]) + bytes([len(nb)]) + nb + struct.pack("<Q", addr)  # 1-byte name length, hard link

    x_at, y_at = dataset(arr), dataset(sub)
    linfo = bytes([0, 0]) + struct.pack("<QQ", h5file.UNDEF, h5file.UNDEF)  # compact storage
    g_at = put(ohdr([msg(0x02, linfo), msg(0x06, link("y", y_at))]))
    # continuation chunk with one more link
    cont_body = msg(0x06, link("g", g_at))
    cont_at = put(b"OCHK" + cont_body + b"\0" * 4)
    attr_name = b"units\0"
    attr_dt = h5file._encode_dtype(np.dtype("<i8"))
    attr_space = bytes([2, 0, 0, 0])  # scalar
    attr = (bytes([3, 0]) + struct.pack("<HHH", len(attr_name), len(attr_dt), len(attr_space)) + bytes([0])
            + attr_name + attr_dt + attr_space + struct.pack("<q", 42))
    root_at = put(ohdr([msg(0x02, linfo), msg(0x06, link("x", x_at)), msg(0x0C, attr),
                        msg(0x10, struct.pack("<QQ", cont_at, len(cont_body) + 8))]))
    eof = len(buf)
    sb = h5file.SIGNATURE + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", 0, h5file.UNDEF, eof, root_at) + b"\0" * 4
    buf[:48] = sb
    with open(path, "wb") as f:
        f.write(bytes(buf))


def test_reader_newer_format(tmp_path):
    rng = np.random.default_rng(9)
    arr, sub = rng.normal(size=(4, 3)), np.arange(7, dtype=np.int64)
    p = tmp_path / "v2.h5"
    _v2_file(p, arr, sub)
    with h5file.File(p) as f:
        assert sorted(f.keys()) == ["g", "x"]
        assert f.attrs["units"] == 42
        assert _eq(np.asarray(f["x"]), arr) and f["x"].extent() is not None
        assert isinstance(f["g"], h5file.Group) and f["g"].keys() == ["y"]
        assert _eq(f["g/y"][...], sub)


def test_loaded_arrays_are_writable():
    got = staging.load(os.path.join(GOLDEN, "staged_rhf.h5"))
    got.ham.h1[0, 0] += 1.0  # h5py hands out writable arrays too
    assert got.ham.chol.flags.writeable and got.trial.data["mo"].flags.writeable


def test_large_string_attributes_and_unicode_names(tmp_path):
    big = "ψ" * 6000 + "end"  # > 4 KB of UTF-8: the global heap collection grows past its minimum
    meta = json.dumps({"basis": "cc-pVTZ", "notes": "x" * 9000})
    p = tmp_path / "u.h5"
    with h5file.File(p, "w") as f:
        f.attrs["meta_json"] = meta
        g = f.create_group("données")
        g.attrs["big"] = big
        g.attrs["small"] = "ok"
        g.create_dataset("énergie", data=np.arange(3.0))
    with h5file.File(p) as f:
        assert f.attrs["meta_json"] == meta
        g = f["données"]
        assert g.attrs["big"] == big and g.attrs["small"] == "ok"
        assert _eq(g["énergie"][...], np.arange(3.0))
