"""NPY / NPZ straight to and from device memory (io::npy_npz,
src/io/npy_npz.rs).

CPU tests parse headers and ZIP directories through the library (no GPU is
touched: nrs_npy_inspect / nrs_npz_locate take a NULL handle) against files
numpy writes, and pin the oracle's header rules to the reference's own test
literals. GPU tests move payloads both ways and compare bit for bit.
"""
import zipfile

import numpy as np
import pytest

from oracle import npy as ON


def _lib():
    from numrs_gb300 import _lib as L
    return L


def _inspect(path, offset=0):
    from numrs_gb300 import kernels as K
    return K.npy_info(path, offset)


def _numpy_header_len(path):
    with open(path, "rb") as f:
        major, _ = np.lib.format.read_magic(f)
        if major == 1:
            np.lib.format.read_array_header_1_0(f)
        else:
            np.lib.format.read_array_header_2_0(f)
        return f.tell()


# -- oracle pinned to the reference's tests -----------------------------------
def test_oracle_header_matches_reference_tests():
    # test_npy_header_construction / test_npy_header_parsing
    # (src/io/npy_npz.rs:714-742)
    h = ON.construct_npy_header("<f4", [2, 3])
    assert h[:6] == b"\x93NUMPY" and h[6] == 1 and h[7] == 0
    text = h[10:].decode()
    assert "'shape': (2, 3)" in text and "'descr': '<f4'" in text
    assert "'fortran_order': False" in text
    assert ON.parse_npy_header(h) == ([2, 3], "<f4")
    assert len(h) % 16 == 0
    # 1-D tuples carry a trailing comma; a scalar has ()
    assert "'shape': (5,)" in ON.construct_npy_header("<f8", [5]).decode("latin1")
    assert "'shape': ()" in ON.construct_npy_header("<i8", []).decode("latin1")


@pytest.mark.parametrize("shape", [(2, 3), (5,), (), (1, 2, 3, 4), (0,), (7, 0, 3)])
def test_numpy_reads_reference_headers(tmp_path, shape):
    a = np.arange(int(np.prod(shape)), dtype=np.float32).reshape(shape)
    p = tmp_path / "r.npy"
    p.write_bytes(ON.construct_npy_header("<f4", shape) + a.tobytes())
    b = np.load(p)
    assert b.shape == a.shape and np.array_equal(a, b)


# -- header / directory parsing through the library (CPU) ----------------------
@pytest.mark.parametrize("dtype", ["<f4", "<f8", "<i4", "<i8", "<u1", "|b1", "<i2"])
@pytest.mark.parametrize("shape", [(3, 4), (10,), (), (2, 3, 5), (0, 4)])
def test_inspect_numpy_files(tmp_path, dtype, shape):
    a = np.zeros(shape, dtype=np.dtype(dtype))
    p = tmp_path / "a.npy"
    np.save(p, a)
    info = _inspect(p)
    assert info["descr"] == np.dtype(dtype).str
    assert info["shape"] == tuple(shape)
    assert info["itemsize"] == np.dtype(dtype).itemsize
    assert info["data_offset"] == _numpy_header_len(p)
    assert info["nbytes"] == a.nbytes
    assert not info["fortran_order"]
    L = _lib()
    want = {"<f4": L.F32, "<f8": L.F64, "<i4": L.I32, "<i8": L.I64}.get(dtype, -1)
    assert info["dtype"] == want


def test_inspect_reference_header(tmp_path):
    p = tmp_path / "r.npy"
    hdr = ON.construct_npy_header("<f8", [3, 2])
    p.write_bytes(hdr + np.zeros(6).tobytes())
    info = _inspect(p)
    assert info["shape"] == (3, 2) and info["descr"] == "<f8" and info["data_offset"] == len(hdr) == 80


def test_inspect_flags_and_errors(tmp_path):
    L = _lib()
    p = tmp_path / "f.npy"
    np.save(p, np.asfortranarray(np.zeros((3, 4))))
    assert _inspect(p)["fortran_order"]
    bad = tmp_path / "bad.npy"
    bad.write_bytes(b"NOTNPY" + b"\0" * 100)
    with pytest.raises(L.NumRs2Error) as e:
        _inspect(bad)
    assert e.value.status == L.ERR_INVALID
    v2 = tmp_path / "v2.npy"
    with open(v2, "wb") as f:
        np.lib.format.write_array(f, np.zeros(4), version=(2, 0))
    with pytest.raises(L.NumRs2Error) as e:
        _inspect(v2)
    assert e.value.status == L.ERR_UNSUPPORTED
    short = tmp_path / "short.npy"
    np.save(short, np.zeros(1000))
    data = short.read_bytes()
    short.write_bytes(data[:-8])
    with pytest.raises(L.NumRs2Error):
        _inspect(short)
    with pytest.raises(L.NumRs2Error) as e:
        _inspect(tmp_path / "missing.npy")
    assert e.value.status == L.ERR_IO


def _locate(path, name):
    import ctypes as C
    L = _lib()
    off, size = C.c_int64(), C.c_int64()
    L.check(L.load().nrs_npz_locate(None, str(path).encode(), None if name is None else name.encode(),
                                    C.byref(off), C.byref(size)))
    return off.value, size.value


def test_npz_locate(tmp_path):
    L = _lib()
    a = np.arange(12, dtype=np.float32).reshape(3, 4)
    b = np.arange(5, dtype=np.int64)
    p = tmp_path / "s.npz"
    np.savez(p, first=a, second=b)
    for name, arr in (("first", a), ("second", b), (None, a)):
        off, size = _locate(p, name)
        info = _inspect(p, off)
        assert info["shape"] == arr.shape and info["descr"] == arr.dtype.str
        raw = p.read_bytes()[info["data_offset"]:info["data_offset"] + info["nbytes"]]
        assert np.array_equal(np.frombuffer(raw, dtype=arr.dtype).reshape(arr.shape), arr)
        assert size == info["data_offset"] - off + info["nbytes"]
    with pytest.raises(L.NumRs2Error):
        _locate(p, "third")
    c = tmp_path / "c.npz"
    np.savez_compressed(c, x=a)
    with pytest.raises(L.NumRs2Error) as e:
        _locate(c, "x")
    assert e.value.status == L.ERR_UNSUPPORTED
    # a ZIP with an archive comment and no .npy member
    z = tmp_path / "z.npz"
    with zipfile.ZipFile(z, "w") as zf:
        zf.writestr("readme.txt", "x")
        zf.comment = b"c" * 300
    with pytest.raises(L.NumRs2Error):
        _locate(z, None)


# -- payloads through the GPU ---------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("dtype,shape", [(np.float32, (3, 5)), (np.float64, (1000, 1001)),
                                         (np.int64, (7,)), (np.int32, ()), (np.float32, (0, 3)),
                                         (np.float32, (9000, 1000 + 7))])
def test_load_numpy_files_bit_exact(K, tmp_path, dtype, shape):
    r = np.random.default_rng(1)
    a = np.asarray((r.standard_normal(shape) * 1e3).astype(dtype))
    p = tmp_path / "a.npy"
    np.save(p, a)
    t = K.load_npy(p)
    assert tuple(t.shape) == a.shape
    got = t.cpu().numpy()
    assert got.tobytes() == a.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,shape", [(np.float32, (3, 5)), (np.float64, (4097,)), (np.int64, ()),
                                         (np.int32, (2, 3, 4)), (np.float32, (0,)),
                                         (np.float32, (5000, 4000 + 3))])
def test_save_matches_reference_writer(K, tmp_path, dtype, shape):
    import torch
    r = np.random.default_rng(2)
    a = np.asarray((r.standard_normal(shape) * 1e3).astype(dtype))
    p = tmp_path / "s.npy"
    K.save_npy(p, torch.from_numpy(a).cuda())
    want = ON.construct_npy_header(np.dtype(dtype).str, list(shape)) + a.tobytes()
    assert p.read_bytes() == want
    b = np.load(p)
    assert b.shape == a.shape and b.tobytes() == a.tobytes()


@pytest.mark.gpu
def test_roundtrip_and_npz(K, tmp_path):
    import torch
    x = torch.empty((2048, 3000), device="cuda")
    K.fill_random(x, _lib().RNG_NORMAL, 9, 0.0, 1.0)
    p = tmp_path / "x.npy"
    K.save_npy(p, x)
    y = K.load_npy(p)
    assert torch.equal(x.view(torch.int32), y.view(torch.int32))
    z = tmp_path / "z.npz"
    a = np.arange(30, dtype=np.float64).reshape(5, 6)
    np.savez(z, a=a, x=x.cpu().numpy())
    assert torch.equal(K.load_npz(z, "x").view(torch.int32), x.view(torch.int32))
    assert np.array_equal(K.load_npz(z).cpu().numpy(), a)
    with pytest.raises(_lib().NumRs2Error):
        K.save_npy(p, x.t())
