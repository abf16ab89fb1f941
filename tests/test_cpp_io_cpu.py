"""HDF5 input files of the C++ binary (``kwave_gb300.h5io``,
``kwave_gb300.cpp_io``), on the CPU.

* The file container: round trips of float32/float64/integer datasets of
  every rank (scalars, empty, contiguous and chunked), string attributes on
  datasets and on the root group, groups of more names than one symbol table
  node holds; the structure of the written bytes (superblock version 0,
  8-byte offsets, end-of-file address, B-tree and node signatures).
* The content: ``kspaceFirstOrder(..., backend="gb300", save_only=True)``
  writes the datasets the unmodified reference writes with
  ``backend="cpp"`` (goldens captured from kwave/solvers/cpp_simulation.py
  by ``tests/golden/make_cpp_io_golden.py``): same names, shapes, dtypes,
  values and attributes; read back from the file.
* The way back: the problem read from such a file is the problem the native
  solver runs for the same call (grids, masks, source rows in C order, p0).
"""
import struct
import sys
from pathlib import Path
from types import SimpleNamespace as NS

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))

from fixtures import load_case  # noqa: E402

from kwave_gb300 import cpp_io, h5io, unified  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "cpp_io"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


def test_round_trip_container(tmp_path):
    rng = np.random.default_rng(0)
    ds = {f"d{i:02d}": rng.standard_normal((1, 3, i + 1)).astype(np.float32) for i in range(45)}
    ds.update(Nx=np.array([[[128]]], dtype=np.uint64), big=rng.standard_normal((4, 5, 6)),
              ints=rng.integers(-5, 5, size=(7,)).astype(np.int32), empty=np.zeros((0,), np.float32),
              scalar=np.float32(3.5), chunked=rng.standard_normal((9, 10, 11)).astype(np.float32),
              chunked2=np.arange(60, dtype=np.uint64).reshape(1, 6, 10))
    at = {k: {"data_type": "float", "domain_type": "real"} for k in ds}
    at["Nx"] = {"data_type": "long", "domain_type": "real", "empty": ""}
    root = {"created_by": "k-Wave test", "file_type": "input", "major_version": "1"}
    path = tmp_path / "t.h5"
    h5io.write_file(path, ds, at, root, chunks={"chunked": (4, 3, 5), "chunked2": (1, 4, 4)})
    got, gat, groot = h5io.read_file(path)
    assert set(got) == set(ds)
    for k, v in ds.items():
        v = np.asarray(v)
        assert got[k].dtype == v.dtype and got[k].shape == v.shape and np.array_equal(got[k], v), k
    assert gat == at
    assert groot == root


def test_round_trip_filtered_chunks(tmp_path):
    """Deflated (levels 1, 4, 9) and shuffled chunks, edge chunks included,
    of float32/float64/uint64/int32 datasets of rank 1-3 read back exactly;
    the chunks of compressible data take fewer bytes than the data."""
    rng = np.random.default_rng(3)
    ds = {"f32": rng.standard_normal((9, 10, 11)).astype(np.float32),
          "f64": rng.standard_normal((5, 23)),
          "u64": np.arange(70, dtype=np.uint64).reshape(1, 7, 10),
          "i32": rng.integers(-9, 9, size=(33,)).astype(np.int32),
          "zeros": np.zeros((1, 64, 64), np.float32)}
    chunks = {"f32": (4, 3, 5), "f64": (2, 8), "u64": (1, 4, 4), "i32": (7,), "zeros": (1, 8, 64)}
    comp = {"f32": 1, "f64": 4, "u64": 9, "i32": 6, "zeros": 9}
    path = tmp_path / "z.h5"
    h5io.write_file(path, ds, chunks=chunks, compression=comp, shuffle={"f32", "u64"})
    got, _, _ = h5io.read_file(path)
    for k, v in ds.items():
        assert got[k].dtype == v.dtype and np.array_equal(got[k], v), k
    plain = tmp_path / "p.h5"
    h5io.write_file(plain, {"zeros": ds["zeros"]}, chunks={"zeros": (1, 8, 64)})
    small = tmp_path / "s.h5"
    h5io.write_file(small, {"zeros": ds["zeros"]}, chunks={"zeros": (1, 8, 64)}, compression={"zeros": 9})
    assert small.stat().st_size < plain.stat().st_size - 10000
    with pytest.raises(ValueError, match="chunked"):
        h5io.write_file(tmp_path / "x.h5", {"a": np.zeros(4, np.float32)}, compression={"a": 4})


def test_filter_messages_and_chunk_decoding():
    """The filter pipeline message as the format specification lays it out
    (version 1 written; versions 1 and 2 read), and chunk decoding: filters
    undone last first, a chunk's filter-mask bit skips that filter, the
    Fletcher-32 filter's 4 trailing bytes are stripped."""
    import struct
    import zlib

    msg = h5io._filter_message([(h5io.FILTER_SHUFFLE, [4]), (h5io.FILTER_DEFLATE, [6])])
    assert msg[:2] == bytes([1, 2]) and msg[2:8] == b"\0" * 6
    assert struct.unpack_from("<HHHH", msg, 8) == (2, 0, 0, 1) and struct.unpack_from("<I", msg, 16)[0] == 4
    assert struct.unpack_from("<HHHH", msg, 24) == (1, 0, 0, 1) and struct.unpack_from("<I", msg, 32)[0] == 6
    assert len(msg) == 40  # odd client-data counts padded to 8 bytes in version 1
    assert h5io._parse_filters(msg, 0) == [(2, [4]), (1, [6])]
    v2 = bytes([2, 2]) + struct.pack("<HHHI", 2, 1, 1, 8) + struct.pack("<HHHI", 1, 0, 1, 9)
    assert h5io._parse_filters(v2, 0) == [(2, [8]), (1, [9])]
    raw = np.arange(12, dtype=np.float32).tobytes()
    shuffled = h5io._shuffle(raw, 4)
    assert shuffled != raw and h5io._unshuffle(shuffled, 4) == raw
    pipe = [(h5io.FILTER_SHUFFLE, [4]), (h5io.FILTER_DEFLATE, [5])]
    stored = zlib.compress(shuffled, 5)
    assert h5io._decode_chunk(stored, pipe, 0, 4) == raw
    assert h5io._decode_chunk(zlib.compress(raw), pipe, 0b01, 4) == raw      # shuffle skipped for this chunk
    assert h5io._decode_chunk(raw + b"abcd", [(h5io.FILTER_FLETCHER32, [])], 0, 4) == raw
    with pytest.raises(NotImplementedError, match="filter 4"):
        h5io._decode_chunk(raw, [(4, [])], 0, 4)


def test_container_structure(tmp_path):
    path = tmp_path / "s.h5"
    names = [f"n{i:03d}" for i in range(20)]
    h5io.write_file(path, {n: np.float32(i) for i, n in enumerate(names)})
    b = path.read_bytes()
    assert b[:8] == b"\x89HDF\r\n\x1a\n"
    assert b[8] == 0 and b[13] == 8 and b[14] == 8
    leaf_k, internal_k = struct.unpack_from("<HH", b, 16)
    assert (leaf_k, internal_k) == (h5io.LEAF_K, h5io.INTERNAL_K)
    base, free, eof, drv = struct.unpack_from("<QQQQ", b, 24)
    assert base == 0 and free == h5io.UNDEF and drv == h5io.UNDEF and eof == len(b)
    _, root, cache, btree, heap = struct.unpack_from("<QQI4xQQ", b, 56)
    assert cache == 1 and b[btree:btree + 4] == b"TREE" and b[heap:heap + 4] == b"HEAP"
    ntype, level, used = struct.unpack_from("<BBH", b, btree + 4)
    assert (ntype, level, used) == (0, 0, -(-len(names) // (2 * h5io.LEAF_K)))
    # children in name order, each key after a child is the child's last name
    heap_data = struct.unpack_from("<Q", b, heap + 24)[0]

    def name(off):
        e = b.index(b"\0", heap_data + off)
        return b[heap_data + off:e].decode()

    seen = []
    for i in range(used):
        child, key = struct.unpack_from("<QQ", b, btree + 32 + 16 * i)
        assert b[child:child + 4] == b"SNOD"
        count = struct.unpack_from("<H", b, child + 6)[0]
        here = [name(struct.unpack_from("<Q", b, child + 8 + 40 * j)[0]) for j in range(count)]
        assert here == sorted(here) and name(key) == here[-1]
        seen += here
    assert seen == sorted(names)


def test_refusals(tmp_path):
    with pytest.raises(ValueError):
        h5io.write_file(tmp_path / "x.h5", {"a/b": np.float32(1)})
    (tmp_path / "y.h5").write_bytes(b"not an hdf5 file")
    with pytest.raises(ValueError, match="signature"):
        h5io.read_file(tmp_path / "y.h5")
    with pytest.raises(ValueError, match="single or uint64"):
        cpp_io.matrix(np.zeros((2, 2), np.float64))
    with pytest.raises(ValueError, match="2-D arrays"):
        cpp_io.matrix(np.zeros(5, np.float32))


def _matrix_layout_reference(a):
    """kwave/utils/io.py:64-78 with the reshape h5py applies."""
    if a.ndim == 3:
        m = np.transpose(a, [2, 1, 0])
        return m.reshape(m.shape)
    if a.ndim == 2:
        m = np.transpose(a)
        return m.reshape((1,) + m.shape)
    return a.reshape(1, 1, 1)


def test_matrix_layout():
    rng = np.random.default_rng(1)
    for a in (rng.standard_normal((3, 4, 5)).astype(np.float32), rng.standard_normal((6, 7)).astype(np.float32),
              np.array([9], dtype=np.uint64), np.float32(2.0)):
        a = np.asarray(a)
        m, at = cpp_io.matrix(a)
        assert np.array_equal(m, _matrix_layout_reference(a))
        assert at["domain_type"] == "real"
        back = cpp_io.unmatrix(m, a.ndim if a.ndim >= 2 else 2)
        assert np.array_equal(back, a.reshape(back.shape))


def _golden(name):
    z = np.load(GOLDEN / f"{name}.npz", allow_pickle=False)
    h5 = {k[3:]: z[k] for k in z.files if k.startswith("h5:")}
    at = {}
    for k in z.files:
        if k.startswith("h5attr:"):
            _, ds, a = k.split(":", 2)
            at.setdefault(ds, {})[a] = z[k].tobytes().rstrip(b"\0").decode()
    root = {k[7:]: z[k].tobytes().rstrip(b"\0").decode() for k in z.files if k.startswith("h5root:")}
    ret_pml = tuple(z["meta:ret_pml_size"].tolist()) if "meta:ret_pml_size" in z.files else None
    return h5, at, root, ret_pml


def _call(name, data_path):
    prob, _, _, meta = load_case(name, "cpp_io")
    opts = {k[4:]: (v.item() if v.ndim == 0 else tuple(v.tolist())) for k, v in meta.items() if k.startswith("opt_")}
    import api_cases

    kgrid, medium, source, sensor = api_cases.objects(prob)
    if sensor is not None:
        sensor.record = None
    return unified.kspaceFirstOrder(kgrid, medium, source, sensor, backend="gb300", save_only=True,
                                    data_path=str(data_path), **opts), prob, opts


@pytest.mark.parametrize("name", CASES)
def test_save_only_matches_reference(name, tmp_path):
    """The input file of kspaceFirstOrder(save_only=True) holds what the
    reference's backend='cpp' writes for the same call."""
    ref, ref_at, ref_root, ret_pml = _golden(name)
    res, _, _ = _call(name, tmp_path)
    assert res["input_file"].endswith("kwave_input.h5") and res["output_file"].endswith("kwave_output.h5")
    assert (tuple(res["pml_size"]) if "pml_size" in res else None) == ret_pml
    got, got_at, got_root = h5io.read_file(res["input_file"])
    assert set(got) == set(ref), (sorted(set(got) ^ set(ref)))
    for k, r in ref.items():
        g = got[k]
        assert g.dtype == r.dtype and g.shape == r.shape, (k, g.dtype, r.dtype, g.shape, r.shape)
        if k == "p0_source_input":
            # smoothed in float64 on both sides, then rounded to float32
            d = np.abs(g.astype(np.float64) - r.astype(np.float64))
            assert np.all(d <= np.spacing(np.abs(r).astype(np.float32)).astype(np.float64)), (k, float(d.max()))
        else:
            assert np.array_equal(g, r), (k, g.ravel()[:4], r.ravel()[:4])
        assert got_at[k] == ref_at[k], k
    assert set(got_root) == set(ref_root)
    for a in ("major_version", "minor_version", "file_type"):
        assert got_root[a] == ref_root[a]
    assert got_root["created_by"].startswith("k-Wave ")
    with pytest.raises(FileExistsError):
        _call(name, tmp_path)


@pytest.mark.parametrize("name", CASES)
def test_problem_from_input_file(name, tmp_path):
    """Reading the file back gives the problem the native solver runs for
    the same call: grid, PML, medium, p0, sources (rows in C order of the
    mask's points) and the sensor's grid points."""
    res, prob0, opts = _call(name, tmp_path)
    prob = cpp_io.problem_from_input_file(res["input_file"])
    want, pml = unified.prepare_problem(*__import__("api_cases").objects(prob0), **{
        k: v for k, v in opts.items() if k in ("pml_size", "pml_alpha", "pml_inside", "smooth_p0")})
    shape = tuple(want["shape"])
    assert prob["shape"] == shape and prob["pml_size"] == tuple(pml)
    np.testing.assert_allclose(prob["spacing"], want["spacing"], rtol=1e-7)
    np.testing.assert_allclose(prob["dt"], want["dt"], rtol=1e-7)
    assert prob["Nt"] == want["Nt"]
    for k in ("sound_speed", "density"):
        np.testing.assert_allclose(np.broadcast_to(prob[k], shape), np.broadcast_to(np.asarray(want[k], np.float32),
                                   shape), rtol=0, atol=0)
    if want.get("p0") is not None:
        p0 = np.asarray(want["p0"], dtype=np.float64).reshape(shape)
        if want.get("smooth_p0", True):
            p0 = cpp_io.smooth_host(p0)
        np.testing.assert_array_equal(prob["p0"], p0.astype(np.float32))
    for m, sig in (("p_mask", ("p",)), ("u_mask", ("ux", "uy", "uz"))):
        if want.get(m) is None:
            continue
        assert np.array_equal(prob[m], np.asarray(want[m]).astype(bool).reshape(shape))
        for s in sig:
            if want.get(s) is not None:
                w = np.asarray(want[s], dtype=np.float32)
                w = w.reshape(-1, w.shape[-1])
                assert np.array_equal(prob[s], w), s
    sm = want.get("sensor_mask")
    if sm is None:
        assert prob["sensor_mask"].all()
    elif np.asarray(sm).shape == shape:
        assert np.array_equal(prob["sensor_mask"], np.asarray(sm).astype(bool))
    else:
        from kwave_gb300.conversion import cart2grid

        kg = NS(N=np.array(shape), spacing=np.array(want["spacing"]), dim=len(shape))
        assert np.array_equal(prob["sensor_mask"], cart2grid(kg, np.asarray(sm), order="C")[0].astype(bool))


def test_source_rows_fortran_to_c():
    """The C++ binary pairs signal rows with the Fortran-order index list;
    the native solver with mask points in C order."""
    shape = (4, 5)
    m = np.zeros(shape, bool)
    m[1, 3] = m[2, 1] = m[3, 0] = True
    idx = cpp_io._fortran_index(m, shape)
    rows = np.arange(3)[:, None] * np.ones((1, 6))   # row i belongs to the i-th F-order point
    c = cpp_io._rows_to_c_order(rows, idx, shape)
    f_points = [tuple(p) for p in np.argwhere(m.T)[:, ::-1]]          # F order
    c_points = [tuple(p) for p in np.argwhere(m)]                     # C order
    for i, p in enumerate(c_points):
        assert c[i, 0] == f_points.index(p)


def test_save_only_refusals(tmp_path):
    import api_cases

    prob = dict(shape=(24, 20), spacing=(1e-4, 1e-4), Nt=10, dt=1e-8, sound_speed=1500.0, density=1000.0,
                p0=np.ones((24, 20)))
    kgrid, medium, source, sensor = api_cases.objects(prob)
    with pytest.raises(ValueError, match="data_path must be provided"):
        unified.kspaceFirstOrder(kgrid, medium, source, sensor, save_only=True, pml_size=4, pml_inside=True)
    medium.alpha_coeff, medium.alpha_power, medium.alpha_mode = 0.5, 1.5, "no_dispersion"
    with pytest.raises(ValueError, match="alpha_mode"):
        unified.kspaceFirstOrder(kgrid, medium, source, sensor, save_only=True, data_path=str(tmp_path),
                                 pml_size=4, pml_inside=True)
    with pytest.raises(NotImplementedError, match="binaries"):
        unified.kspaceFirstOrder(kgrid, medium, source, sensor, binary_path="/bin/true", pml_size=4)
