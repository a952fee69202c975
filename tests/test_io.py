"""LSMLIB's binary Grid and data-array files: this library's readers and
writers (include/lsmgpu_io.h) against the reference's own C code
(src/utils/lsm_grid.c, lsm_data_arrays.c, lsm_file.c, compiled into
oracle/_ref/liblsmrefio.so).

Bars: files written by either side are byte-identical; either side reads the
other's files to identical values and Grid members; gzip round trips work both
ways; a short or missing file and a too-small buffer report errors.  The GPU
tests write device arrays and read files straight into device memory.
"""
import ctypes
import os
import shutil

import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

REF_IO = os.path.join(H.ROOT, "oracle", "_ref", "liblsmrefio.so")
GRID_BYTES = 297


class Grid(ctypes.Structure):
    """LSMLIB's Grid (src/utils/lsm_grid.h:43-95, double build)."""
    _fields_ = ([("num_dims", ctypes.c_int)] +
                [(n, ctypes.c_double * 3) for n in ("x_lo", "x_hi", "x_lo_ghostbox", "x_hi_ghostbox")] +
                [("grid_dims", ctypes.c_int * 3), ("grid_dims_ghostbox", ctypes.c_int * 3),
                 ("dx", ctypes.c_double * 3), ("num_gridpts", ctypes.c_int)] +
                [("%s%s_%s" % (a, b, box), ctypes.c_int)
                 for box in ("gb", "fb", "D1_fb", "D2_fb", "D3_fb")
                 for a in ("i", "j", "k") for b in ("lo", "hi")] +
                [("num_nb_levels", ctypes.c_int)] +
                [(m, ctypes.c_ubyte) for m in ("mark_gb", "mark_D1", "mark_D2", "mark_D3", "mark_fb")] +
                [("beta", ctypes.c_double), ("gamma", ctypes.c_double)])


def _sig(lib):
    lib.readGridFromBinaryFile.restype = ctypes.POINTER(Grid)
    lib.readGridFromBinaryFile.argtypes = [ctypes.c_char_p]
    lib.writeGridToBinaryFile.argtypes = [ctypes.POINTER(Grid), ctypes.c_char_p, ctypes.c_int]
    lib.writeDataArray.argtypes = [ctypes.c_void_p, ctypes.POINTER(Grid), ctypes.c_char_p, ctypes.c_int]
    lib.writeDataArrayNoGrid.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_char_p,
                                         ctypes.c_int]
    lib.readDataArray.restype = ctypes.POINTER(ctypes.c_double)
    lib.readDataArray.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_char_p]
    lib.writeDataArray1d.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
    lib.readDataArray1d.restype = ctypes.POINTER(ctypes.c_double)
    lib.readDataArray1d.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_char_p]
    return lib


@pytest.fixture(scope="module")
def ours():
    return _sig(L.lib())


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(REF_IO):
        try:
            from oracle import build as ob
            ob.build_ref_io()
        except Exception:
            pass
    if not os.path.exists(REF_IO):
        pytest.skip("reference file code not available (no reference tree)")
    lib = _sig(ctypes.CDLL(REF_IO, mode=ctypes.RTLD_LOCAL))
    lib.createGridSetDxDyDz.restype = ctypes.POINTER(Grid)
    lib.createGridSetDxDyDz.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                        ctypes.c_int]
    return lib


libc = ctypes.CDLL(None)
libc.free.argtypes = [ctypes.c_void_p]


def make_grid(ref, accuracy=3, dx=(0.05, 0.04, 0.025), lo=(-1.0, -0.6, -0.5), hi=(1.0, 0.6, 0.5)):
    c3 = ctypes.c_double * 3
    g = ref.createGridSetDxDyDz(3, dx[0], dx[1], dx[2], c3(*lo), c3(*hi), accuracy)
    g.contents.beta = 0.15
    g.contents.gamma = 0.3
    g.contents.num_nb_levels = 4
    return g


def grid_bytes(g):
    return bytes(ctypes.string_at(ctypes.addressof(g.contents), ctypes.sizeof(Grid)))


def read(path):
    with open(path, "rb") as f:
        return f.read()


def test_struct_layout_matches_c():
    assert ctypes.sizeof(Grid) == 304  # 297 bytes of members plus C alignment padding


@pytest.mark.parametrize("accuracy", [0, 3])
def test_grid_file_byte_identical_and_read_back(accuracy, ours, ref, tmp_path):
    g = make_grid(ref, accuracy)
    a, b = str(tmp_path / "ref.grid").encode(), str(tmp_path / "ours.grid").encode()
    ref.writeGridToBinaryFile(g, a, 0)
    ours.writeGridToBinaryFile(g, b, 0)
    L.check(ours)
    assert len(read(a)) == GRID_BYTES and read(a) == read(b)
    for reader, path in ((ours, a), (ref, b)):
        r = reader.readGridFromBinaryFile(path)
        # members equal (padding bytes aside): compare field by field
        for name, _ in Grid._fields_:
            va, vb = getattr(r.contents, name), getattr(g.contents, name)
            if hasattr(va, "__len__"):
                assert list(va) == list(vb), name
            else:
                assert va == vb, name
        libc.free(r)
    L.check(ours)


def test_short_and_missing_grid_files(ours, tmp_path):
    p = tmp_path / "short.grid"
    p.write_bytes(b"\x03\x00\x00\x00" + b"\x00" * 10)
    g = ours.readGridFromBinaryFile(str(p).encode())
    assert g.contents.num_dims == 3 and g.contents.num_gridpts == 0
    assert L.last_error(ours)[0] == 3
    libc.free(g)
    g = ours.readGridFromBinaryFile(str(tmp_path / "absent.grid").encode())
    assert g.contents.num_dims == 0 and L.last_error(ours)[0] == 3
    libc.free(g)
    one = np.zeros(1)
    ours.writeDataArray1d(one.ctypes.data, 1, str(tmp_path / "ok.1d").encode(), 0)
    assert L.last_error(ours)[0] == 0


def _arr(n, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal(n))


def test_data_array_byte_identical_and_read_back(ours, ref, tmp_path):
    g = make_grid(ref)
    n = tuple(g.contents.grid_dims_ghostbox)
    assert int(np.prod(n)) == g.contents.num_gridpts
    data = _arr(n, 1)
    a, b = str(tmp_path / "ref.dat").encode(), str(tmp_path / "ours.dat").encode()
    ref.writeDataArray(data.ctypes.data, g, a, 0)
    ours.writeDataArray(data.ctypes.data, g, b, 0)
    L.check(ours)
    assert read(a) == read(b) and len(read(a)) == 12 + 8 * data.size
    for reader, path in ((ours, a), (ref, b)):
        dims = (ctypes.c_int * 3)()
        ptr = reader.readDataArray(dims, path)
        got = np.ctypeslib.as_array(ptr, shape=(data.size,)).copy()
        libc.free(ptr)
        assert tuple(dims) == n
        assert H.same(got, data.ravel(order="F"))


def test_data_array_no_grid_and_1d(ours, ref, tmp_path):
    n = (7, 5, 3)
    data = _arr(n, 2)
    nn = (ctypes.c_int * 3)(*n)
    a, b = str(tmp_path / "ref.nog").encode(), str(tmp_path / "ours.nog").encode()
    ref.writeDataArrayNoGrid(data.ctypes.data, nn, a, 0)
    ours.writeDataArrayNoGrid(data.ctypes.data, nn, b, 0)
    assert read(a) == read(b)
    v = _arr(37, 3)
    a, b = str(tmp_path / "ref.1d").encode(), str(tmp_path / "ours.1d").encode()
    ref.writeDataArray1d(v.ctypes.data, v.size, a, 0)
    ours.writeDataArray1d(v.ctypes.data, v.size, b, 0)
    assert read(a) == read(b)
    for reader, path in ((ours, a), (ref, b)):
        cnt = ctypes.c_int()
        ptr = reader.readDataArray1d(ctypes.byref(cnt), path)
        assert cnt.value == v.size
        assert H.same(np.ctypeslib.as_array(ptr, shape=(v.size,)).copy(), v)
        libc.free(ptr)
    L.check(ours)


@pytest.mark.skipif(shutil.which("gzip") is None, reason="gzip not on PATH")
def test_gzip_round_trips_both_ways(ours, ref, tmp_path):
    n = (6, 4, 5)
    data = _arr(n, 4)
    nn = (ctypes.c_int * 3)(*n)
    for writer, reader in ((ours, ref), (ref, ours)):
        base = str(tmp_path / ("w%d" % id(writer))).encode()
        writer.writeDataArrayNoGrid(data.ctypes.data, nn, base, 1)
        assert os.path.exists(base + b".gz") and not os.path.exists(base)
        dims = (ctypes.c_int * 3)()
        ptr = reader.readDataArray(dims, base + b".gz")
        assert tuple(dims) == n
        assert H.same(np.ctypeslib.as_array(ptr, shape=(data.size,)).copy(), data.ravel(order="F"))
        libc.free(ptr)
        # the reader compresses the file again after reading it
        assert os.path.exists(base + b".gz") and not os.path.exists(base)
    L.check(ours)


def test_read_into_host_buffer_and_capacity(ours, tmp_path):
    n = (4, 3, 2)
    data = _arr(n, 5)
    path = str(tmp_path / "into.dat").encode()
    ours.writeDataArrayNoGrid(data.ctypes.data, (ctypes.c_int * 3)(*n), path, 0)
    fn = ours.lsmgpu_read_data_array_into
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_longlong]
    out = np.full(data.size, -1.0)
    dims = (ctypes.c_int * 3)()
    assert fn(path, dims, out.ctypes.data, 23) == 4  # LSMGPU_ERR_CAPACITY, nothing written
    assert np.all(out == -1.0)
    assert fn(path, dims, out.ctypes.data, out.size) == 0
    assert tuple(dims) == n and H.same(out, data.ravel(order="F"))
    assert fn(str(tmp_path / "absent").encode(), dims, out.ctypes.data, out.size) == 3
    # a file shorter than its header says
    with open(path, "r+b") as f:
        f.truncate(12 + 8 * 5)
    assert fn(path, dims, out.ctypes.data, out.size) == 3
    # a valid call clears the status
    ours.writeDataArrayNoGrid(data.ctypes.data, (ctypes.c_int * 3)(*n), path, 0)
    assert L.last_error(ours)[0] == 0


@pytest.mark.gpu
def test_device_arrays_write_and_read(ours, tmp_path):
    import torch
    n = (130, 97, 64)          # within one 32 MB pinned chunk
    big = (262, 256, 130)      # 70 MB: three chunks
    for shape in (n, big):
        host = np.asfortranarray(np.random.default_rng(6).standard_normal(shape))
        dev = torch.from_numpy(np.ascontiguousarray(host.T)).cuda()
        a, b = str(tmp_path / "h.dat").encode(), str(tmp_path / "d.dat").encode()
        nn = (ctypes.c_int * 3)(*shape)
        ours.writeDataArrayNoGrid(host.ctypes.data, nn, a, 0)
        ours.writeDataArrayNoGrid(dev.data_ptr(), nn, b, 0)
        L.check(ours)
        assert read(a) == read(b)
        back = torch.full_like(dev, -1.0)
        fn = ours.lsmgpu_read_data_array_into
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_longlong]
        dims = (ctypes.c_int * 3)()
        assert fn(b, dims, back.data_ptr(), back.numel()) == 0
        assert tuple(dims) == shape
        assert torch.equal(back, dev)
