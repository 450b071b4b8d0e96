"""Map ingest from the reference's HDF5 file layout (CPU): the reader against
files written byte by byte from the HDF5 file format specification
(tests/h5_files.py), in both the earliest format (superblock 0, symbol-table
groups, version 1 object headers: the reference's case) and the latest
(superblock 2, compact link messages, version 2 object headers).

No map file written by the reference exists on this machine.  The one file
here that the HDF5 library itself wrote (SciPy's MATLAB 7.3 test file) pins
the structures the library writes by default, which are those of the
reference's map files: the reader walks it and finds its dataset's type,
shape, storage and values.  The "/map" layout itself rests on the reference's
writer code (global_map.cpp)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import h5_files as H
from tsdf_localization_gb300 import TsdflError, build_map_codes, read_map_h5, synth
from tsdf_localization_gb300 import _native as N


def _chunks(names, edge, seed):
    rng = np.random.default_rng(seed)
    return {nm: H.Dataset(rng.integers(0, 2**32, size=edge ** 3, dtype=np.uint64).astype(np.uint32))
            for nm in names}


def _expected(chunks):
    names = sorted(chunks, key=lambda s: s.encode())   # the group's listing order
    pos = np.array([[int(t) for t in nm.split("_")] for nm in names], np.int32).reshape(-1, 3)
    raw = np.stack([chunks[nm].values for nm in names]) if names else np.zeros((0, 0), np.uint32)
    return pos, raw


NAMES = ["0_0_0", "1_0_0", "10_0_0", "2_0_0", "-1_0_2", "0_-3_1", "3_3_3", "0_1_0", "1_1_1", "-2_-2_-2",
         "5_0_-1", "0_0_1", "4_4_0", "7_1_2", "0_2_2", "1_2_3", "6_6_6", "-1_-1_0", "2_2_0", "9_9_1"]


@pytest.mark.parametrize("fmt,superblock", [("v0", 0), ("v0", 1), ("v2", 2), ("v2", 3)])
@pytest.mark.parametrize("userblock", [0, 512])
def test_reads_chunks_in_listing_order(tmp_path, fmt, superblock, userblock):
    chunks = _chunks(NAMES, 4, 1)
    path = tmp_path / f"map_{fmt}.h5"
    # small B-tree nodes (4 symbols per leaf, 4 children per node): a two-level tree
    H.write(path, chunks, fmt=fmt, leaf_k=2, internal_k=2, userblock=userblock, superblock=superblock)
    pos, raw, edge = read_map_h5(path)
    epos, eraw = _expected(chunks)
    assert edge == 4
    assert np.array_equal(pos, epos)
    assert np.array_equal(raw, eraw)


@pytest.mark.parametrize("fmt", ["v0", "v2"])
def test_storage_variants(tmp_path, fmt):
    """Compact layout, big-endian integers, headers continued in another block,
    storage never written (the fill value, given or default 0)."""
    rng = np.random.default_rng(2)
    v = [rng.integers(0, 2**32, size=8, dtype=np.uint64).astype(np.uint32) for _ in range(5)]
    chunks = {
        "0_0_0": H.Dataset(v[0], layout="compact"),
        "0_0_1": H.Dataset(v[1], big_endian=True),
        "0_1_0": H.Dataset(v[2], split_header=True),
        "1_0_0": H.Dataset(v[3], unwritten=True, fill=0x00050003),
        "1_1_1": H.Dataset(v[4], unwritten=True),
    }
    path = tmp_path / "variants.h5"
    H.write(path, chunks, fmt=fmt)
    pos, raw, edge = read_map_h5(path)
    assert edge == 2
    assert np.array_equal(pos, [[0, 0, 0], [0, 0, 1], [0, 1, 0], [1, 0, 0], [1, 1, 1]])
    assert np.array_equal(raw[0], v[0]) and np.array_equal(raw[1], v[1]) and np.array_equal(raw[2], v[2])
    assert np.all(raw[3] == 0x00050003) and np.all(raw[4] == 0)


def test_map_from_file_equals_map_from_arrays(tmp_path):
    """createTSDFMap through the file: the same coefficients, brick table, slot
    codes and free cells as from the chunk arrays in the reference's visiting
    order."""
    w = synth.World(synth.ROOM, 4)
    chunk_pos, raw = w.tsdf_chunks(64, edge=16)
    names = ["%d_%d_%d" % tuple(p) for p in chunk_pos]
    chunks = {nm: H.Dataset(raw[i]) for i, nm in enumerate(names)}
    path = tmp_path / "room.h5"
    H.write(path, chunks)
    pos, cells, edge = read_map_h5(path)
    order = sorted(range(len(names)), key=lambda i: names[i].encode())
    assert np.array_equal(pos, chunk_pos[order]) and np.array_equal(cells, raw[order])
    a = build_map_codes(pos, cells, edge, 64)
    b = build_map_codes(chunk_pos[order], raw[order], 16, 64)
    for fa, fb in ((a[0], b[0]),):
        assert all(getattr(fa, k) == getattr(fb, k) for k, _ in N.MapCoef._fields_)
    for xa, xb in zip(a[1:], b[1:]):
        assert np.array_equal(xa, xb)


def _code(exc):
    return exc.value.code


def test_unsupported_storage(tmp_path):
    p = tmp_path / "x.h5"
    H.write(p, {"0_0_0": H.Dataset(np.zeros(8, np.uint32), layout="chunked")})
    with pytest.raises(TsdflError) as e:
        read_map_h5(p)
    assert _code(e) == N.TSDFL_ERR_UNSUPPORTED and "chunked" in str(e.value)
    H.write(p, {"0_0_0": H.Dataset(np.zeros(8, np.uint32), filtered=True)})
    with pytest.raises(TsdflError) as e:
        read_map_h5(p)
    assert _code(e) == N.TSDFL_ERR_UNSUPPORTED and "filtered" in str(e.value)
    H.write(p, {"0_0_0": H.Dataset(np.zeros(8, np.uint32))}, fmt="v2", dense_group=True)
    with pytest.raises(TsdflError) as e:
        read_map_h5(p)
    assert _code(e) == N.TSDFL_ERR_UNSUPPORTED and "dense" in str(e.value)


def test_malformed_files(tmp_path):
    p = tmp_path / "x.h5"
    ok = {"0_0_0": H.Dataset(np.arange(8, dtype=np.uint32)), "1_0_0": H.Dataset(np.arange(8, dtype=np.uint32))}
    cases = []
    H.write(p, ok, group_name="grid")
    cases.append(("no /map", p.read_bytes(), 'no object "map"'))
    H.write(p, {"1_2": H.Dataset(np.arange(8, dtype=np.uint32))})
    cases.append(("two parts", p.read_bytes(), "is not <x>_<y>_<z>"))
    H.write(p, {"a_0_0": H.Dataset(np.arange(8, dtype=np.uint32))})
    cases.append(("not a number", p.read_bytes(), "is not <x>_<y>_<z>"))
    H.write(p, {"0_0_0": H.Dataset(np.arange(8, dtype=np.uint32)), "0_0_1": H.Dataset(np.arange(27, dtype=np.uint32))})
    cases.append(("sizes differ", p.read_bytes(), "another size"))
    H.write(p, {"0_0_0": H.Dataset(np.arange(10, dtype=np.uint32))})
    cases.append(("not a cube", p.read_bytes(), "not cubes"))
    H.write(p, ok)
    full = p.read_bytes()
    cases.append(("truncated", full[: len(full) // 2], ""))
    cases.append(("not HDF5", b"CDF\x01" + b"\0" * 200, "not an HDF5 file"))
    for what, data, msg in cases:
        p.write_bytes(data)
        with pytest.raises(TsdflError) as e:
            read_map_h5(p)
        assert _code(e) == N.TSDFL_ERR_INVALID_ARG, what
        assert msg in str(e.value), (what, str(e.value))
    with pytest.raises(TsdflError) as e:
        read_map_h5(tmp_path / "missing.h5")
    assert _code(e) == N.TSDFL_ERR_INVALID_ARG


def test_tag_parsing_follows_stoi(tmp_path):
    """Each part converts as std::stoi does: leading blanks and a sign, digits,
    the rest of the part ignored (map_util.h:28-40)."""
    p = tmp_path / "x.h5"
    H.write(p, {" 7_+2_-3x": H.Dataset(np.arange(8, dtype=np.uint32))})
    pos, _, _ = read_map_h5(p)
    assert pos.tolist() == [[7, 2, -3]]
    H.write(p, {"99999999999_0_0": H.Dataset(np.arange(8, dtype=np.uint32))})
    with pytest.raises(TsdflError):
        read_map_h5(p)


def test_empty_map_group(tmp_path):
    p = tmp_path / "x.h5"
    H.write(p, {})
    pos, raw, edge = read_map_h5(p)
    assert pos.shape == (0, 3) and raw.shape[0] == 0 and edge == 0


@pytest.mark.parametrize("fmt", ["v0", "v2"])
def test_corrupted_files_fail_cleanly(tmp_path, fmt):
    """Random byte corruptions of a valid file: every read either succeeds or
    raises TsdflError (never crashes, hangs or returns garbage shapes)."""
    p = tmp_path / "x.h5"
    H.write(p, _chunks(NAMES[:9], 2, 3), fmt=fmt, leaf_k=2, internal_k=2)
    good = p.read_bytes()
    rng = np.random.default_rng(17)
    for trial in range(300):
        data = bytearray(good)
        for _ in range(int(rng.integers(1, 6))):
            i = int(rng.integers(0, len(data)))
            data[i] = int(rng.integers(0, 256)) if trial % 3 else data[i] ^ 0xFF
        p.write_bytes(bytes(data))
        try:
            pos, raw, edge = read_map_h5(p)
        except TsdflError as e:
            assert e.code in (N.TSDFL_ERR_INVALID_ARG, N.TSDFL_ERR_UNSUPPORTED, N.TSDFL_ERR_OUT_OF_MEMORY)
            continue
        assert pos.shape == (raw.shape[0], 3) and (raw.shape[0] == 0 or raw.shape[1] == edge ** 3)


def test_lookup3_known_values():
    """The checksum the test files carry is lookup3's hashlittle: the values
    its author published with the function."""
    assert H.lookup3(b"", 0) == 0xDEADBEEF
    assert H.lookup3(b"", 0xDEADBEEF) == 0xBD5B7DDE
    assert H.lookup3(b"Four score and seven years ago", 0) == 0x17770551
    assert H.lookup3(b"Four score and seven years ago", 1) == 0xCD628161


@pytest.mark.parametrize("superblock", [2, 3])
@pytest.mark.parametrize("where", ["superblock", "object header", "continuation"])
def test_version2_checksums_verified(tmp_path, superblock, where):
    """A byte changed inside a checksummed version 2 structure is reported
    (TSDFL_ERR_INVALID_ARG); the intact file reads."""
    chunks = {"0_0_0": H.Dataset(np.arange(8, dtype=np.uint32), split_header=True),
              "0_0_1": H.Dataset(np.arange(8, 16, dtype=np.uint32))}
    path = tmp_path / "v2.h5"
    H.write(path, chunks, fmt="v2", superblock=superblock)
    pos, raw, edge = read_map_h5(path)
    assert edge == 2 and np.array_equal(raw[1], np.arange(8, 16))
    data = bytearray(path.read_bytes())
    if where == "superblock":
        at = 20    # inside the base / extension addresses
    else:
        sig = b"OHDR" if where == "object header" else b"OCHK"
        at = data.index(sig) + 6
    data[at] ^= 0x40
    bad = tmp_path / "bad.h5"
    bad.write_bytes(bytes(data))
    with pytest.raises(TsdflError) as e:
        read_map_h5(bad)
    assert e.value.code == N.TSDFL_ERR_INVALID_ARG and "checksum" in str(e.value)


ROOT = Path(__file__).resolve().parent.parent


def _libhdf5_file():
    """SciPy's MATLAB 7.3 test file, written by the HDF5 library: a 512-byte
    MATLAB header as the user block, then the library's default structures
    (superblock 0, a symbol-table root group, version 1 object headers, a
    contiguous dataset).  Its one variable is SciPy's ``testdouble`` case,
    pi/4 * (0..8) as a 1x9 double (scipy/io/matlab/tests/test_mio.py)."""
    mio = pytest.importorskip("scipy.io.matlab")
    p = Path(mio.__file__).parent / "tests" / "data" / "testhdf5_7.4_GLNX86.mat"
    if not p.exists():
        pytest.skip("SciPy's HDF5 test file is not installed")
    return p


def test_reader_walks_a_file_written_by_libhdf5(tmp_path):
    src = _libhdf5_file()
    exe = tmp_path / "h5_walk"
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", str(ROOT / "include"),
                    "-I", str(ROOT / "tsdf_localization_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "h5_walk.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(src)], capture_output=True, text=True, check=True).stdout.splitlines()
    links = [ln.split() for ln in out if ln.startswith("link ")]
    assert len(links) == 1, out
    f = links[0]
    assert f[1] == "testdouble", out
    got = dict(zip(f[2::2], f[3::2]))
    # floating point, 8 bytes, little-endian; MATLAB's 1x9 stored column-major as 9x1
    assert (got["class"], got["elem"], got["order"], got["dims"]) == ("1", "8", "le", "9,1"), out
    data = src.read_bytes()
    at = int(got["address"])
    assert at >= 512   # addresses are relative to the superblock after the user block
    values = np.frombuffer(data[at:at + 72], "<f8")
    assert np.array_equal(values, np.pi / 4 * np.arange(9, dtype=float))
    # the map entry point reads the same file and reports the missing group
    status = [ln for ln in out if ln.startswith("map ")][0].split(maxsplit=4)
    assert int(status[1]) == N.TSDFL_ERR_INVALID_ARG and 'no object "map"' in status[4], out
