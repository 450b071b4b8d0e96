"""Small HDF5 files in the layouts the reference's map files take, written
byte by byte for the map reader's tests (there is no HDF5 library here).

Structures follow the HDF5 file format specification:
- "v0": superblock version 0, groups as symbol tables (version 1 B-tree of
  group nodes, local heap, symbol table nodes), version 1 object headers --
  what the HDF5 library writes with its default (earliest) format settings,
  the reference's case (HighFive with default property lists);
- "v2": superblock version 2, version 2 object headers, groups with compact
  link messages -- the latest-format settings.
Datasets are 1-D 4-byte integers, stored contiguously by default.  Version 2
structures carry the format's metadata checksum: Bob Jenkins' lookup3
hashlittle (2006) of the structure's bytes with initial value 0.
"""
from __future__ import annotations

import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"


def lookup3(data: bytes, init: int = 0) -> int:
    """lookup3's hashlittle (Jenkins 2006) of data, 32-bit."""
    M = 0xFFFFFFFF

    def rot(x, r):
        return ((x << r) | (x >> (32 - r))) & M

    n = len(data)
    a = b = c = (0xDEADBEEF + n + init) & M
    k = 0
    while n - k > 12:
        a = (a + int.from_bytes(data[k:k + 4], "little")) & M
        b = (b + int.from_bytes(data[k + 4:k + 8], "little")) & M
        c = (c + int.from_bytes(data[k + 8:k + 12], "little")) & M
        a = (a - c) & M; a ^= rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 4); b = (b + a) & M
        k += 12
    rest = data[k:]
    if not rest:
        return c
    a = (a + int.from_bytes(rest[0:4], "little")) & M
    b = (b + int.from_bytes(rest[4:8], "little")) & M
    c = (c + int.from_bytes(rest[8:12], "little")) & M
    c ^= b; c = (c - rot(b, 14)) & M
    a ^= c; a = (a - rot(c, 11)) & M
    b ^= a; b = (b - rot(a, 25)) & M
    c ^= b; c = (c - rot(b, 16)) & M
    a ^= c; a = (a - rot(c, 4)) & M
    b ^= a; b = (b - rot(a, 14)) & M
    c ^= b; c = (c - rot(b, 24)) & M
    return c


def _sealed(body: bytes) -> bytes:
    """A version 2 structure: its bytes followed by their checksum."""
    return body + struct.pack("<I", lookup3(body))


class Dataset:
    """One dataset: values (uint32 array) and how to store them."""

    def __init__(self, values, big_endian=False, layout="contiguous", split_header=False, unwritten=False,
                 fill=None, filtered=False):
        self.values = np.asarray(values, dtype=np.uint32)
        self.big_endian = big_endian
        self.layout = layout            # "contiguous", "compact", "chunked"
        self.split_header = split_header  # part of the header in a continuation block
        self.unwritten = unwritten      # no storage allocated: the fill value
        self.fill = fill
        self.filtered = filtered


class _Buf:
    def __init__(self, reserve: int):
        self.b = bytearray(reserve)

    def add(self, data: bytes, align: int = 8) -> int:
        self.b += b"\0" * ((-len(self.b)) % align)
        off = len(self.b)
        self.b += data
        return off

    def put(self, off: int, data: bytes) -> None:
        self.b[off:off + len(data)] = data


def _pad8(d: bytes) -> bytes:
    return d + b"\0" * ((-len(d)) % 8)


def _dtype_msg(big_endian: bool) -> bytes:
    # class 0 (fixed point), version 1; bit 0 of the first field byte: byte order
    return struct.pack("<BBBBIHH", 0x10, 1 if big_endian else 0, 0, 0, 4, 0, 32)


def _data_bytes(ds: Dataset) -> bytes:
    return ds.values.astype(">u4" if ds.big_endian else "<u4").tobytes()


def _layout_msg(ds: Dataset, w: _Buf) -> bytes:
    raw = _data_bytes(ds)
    if ds.layout == "compact":
        return struct.pack("<BBH", 3, 0, len(raw)) + raw
    if ds.layout == "chunked":   # version 3, class 2: rank + 1, B-tree address, chunk dims, element size
        return struct.pack("<BBBQII", 3, 2, 2, UNDEF, len(ds.values), 4)
    addr = UNDEF if ds.unwritten else w.add(raw)
    return struct.pack("<BBQQ", 3, 1, addr, len(raw))


def _dataset_msgs(ds: Dataset, w: _Buf, v2: bool) -> list[tuple[int, bytes]]:
    n = len(ds.values)
    space = struct.pack("<BBBBQ", 2, 1, 0, 1, n) if v2 else struct.pack("<BBBB4xQ", 1, 1, 0, 0, n)
    if ds.fill is None:
        fill = struct.pack("<BB", 3, 0x0A) if v2 else struct.pack("<BBBB", 2, 2, 2, 0)
    else:
        fill = (struct.pack("<BBI", 3, 0x2A, 4) if v2 else struct.pack("<BBBBI", 2, 2, 2, 1, 4)) + \
            struct.pack("<I", ds.fill)
    msgs = [(0x01, space), (0x03, _dtype_msg(ds.big_endian)), (0x05, fill)]
    if ds.filtered:   # filter pipeline version 2 with one filter (deflate, level 6)
        msgs.append((0x0B, struct.pack("<BBHHH", 2, 1, 1, 0, 1) + struct.pack("<I", 6)))
    msgs.append((0x08, _layout_msg(ds, w)))
    return msgs


def _v1_block(msgs) -> bytes:
    body = b""
    for t, d in msgs:
        d = _pad8(d)
        body += struct.pack("<HHB3x", t, len(d), 0) + d
    return body


def _v1_header(w: _Buf, msgs, split=False) -> int:
    if split and len(msgs) > 1:
        tail = _v1_block(msgs[1:])
        cont = w.add(tail)
        head = _v1_block(msgs[:1] + [(0x10, struct.pack("<QQ", cont, len(tail)))])
    else:
        head = _v1_block(msgs)
    pre = struct.pack("<BBHII", 1, 0, len(msgs) + (1 if split else 0), 1, len(head)) + b"\0" * 4
    return w.add(pre + head)


def _v2_block(msgs) -> bytes:
    return b"".join(struct.pack("<BHB", t, len(d), 0) + d for t, d in msgs)


def _v2_header(w: _Buf, msgs, split=False) -> int:
    if split and len(msgs) > 1:
        tail = _sealed(b"OCHK" + _v2_block(msgs[1:]))
        cont = w.add(tail)
        body = _v2_block(msgs[:1] + [(0x10, struct.pack("<QQ", cont, len(tail)))])
    else:
        body = _v2_block(msgs)
    body += b"\0\0"   # a gap shorter than a message prefix
    flags = 0x01      # chunk-0 size in 2 bytes
    return w.add(_sealed(b"OHDR" + struct.pack("<BBH", 2, flags, len(body)) + body))


def _symbol_group(w: _Buf, children: dict[str, int], leaf_k: int, internal_k: int) -> tuple[int, int, int]:
    """A group as a symbol table: (object header, B-tree, local heap)."""
    names = sorted(children, key=lambda s: s.encode())
    data = bytearray(b"\0" * 8)   # offset 0: the empty name of the first key
    offs = {}
    for nm in names:
        offs[nm] = len(data)
        data += nm.encode() + b"\0"
    data += b"\0" * ((-len(data)) % 8)
    seg = w.add(bytes(data))
    heap = w.add(b"HEAP" + struct.pack("<B3xQQQ", 0, len(data), UNDEF, seg))
    cap = 2 * leaf_k
    leaves = []   # (address, heap offset of the last name)
    for i in range(0, max(len(names), 1), cap):
        part = names[i:i + cap]
        body = b"SNOD" + struct.pack("<BBH", 1, 0, len(part))
        for nm in part:
            body += struct.pack("<QQII16x", offs[nm], children[nm], 0, 0)
        body += b"\0" * (40 * (cap - len(part)))
        leaves.append((w.add(body), offs[part[-1]] if part else 0))
    level, nodes = 0, leaves
    while True:
        fan = 2 * internal_k
        parents = []
        for i in range(0, len(nodes), fan):
            part = nodes[i:i + fan]
            body = b"TREE" + struct.pack("<BBHQQ", 0, level, len(part), UNDEF, UNDEF)
            body += struct.pack("<Q", 0)
            for addr, last in part:
                body += struct.pack("<QQ", addr, last)
            parents.append((w.add(body), part[-1][1]))   # key 0, then (child i, key i + 1)
        if len(parents) == 1:
            root_tree = parents[0][0]
            break
        nodes, level = parents, level + 1
    header = _v1_header(w, [(0x11, struct.pack("<QQ", root_tree, heap))])
    return header, root_tree, heap


def _link_group(w: _Buf, children: dict[str, int], dense=False) -> int:
    msgs = [(0x02, struct.pack("<BBQQ", 0, 0, 0x1000 if dense else UNDEF, UNDEF)), (0x0A, struct.pack("<BB", 0, 0))]
    for nm, addr in children.items():   # insertion order: the reader sorts by name
        b = nm.encode()
        msgs.append((0x06, struct.pack("<BBB", 1, 0, len(b)) + b + struct.pack("<Q", addr)))
    return _v2_header(w, msgs)


def write(path, chunks: dict[str, Dataset], fmt: str = "v0", leaf_k: int = 4, internal_k: int = 16,
          userblock: int = 0, extra_groups: bool = True, group_name: str = "map", dense_group: bool = False,
          superblock: int | None = None) -> None:
    """A map file: group /<group_name> with one dataset per chunk name (in the
    dict's order), and an unrelated /poses group.  superblock: version 0 or 1
    for fmt "v0", 2 or 3 for fmt "v2"."""
    sbv = superblock if superblock is not None else (0 if fmt == "v0" else 2)
    w = _Buf(100 if fmt == "v0" else 48)
    v2 = fmt == "v2"
    headers = {}
    for nm, ds in chunks.items():
        msgs = _dataset_msgs(ds, w, v2)
        headers[nm] = (_v2_header if v2 else _v1_header)(w, msgs, split=ds.split_header)
    pose = Dataset(np.arange(7, dtype=np.uint32))
    pose_hdr = (_v2_header if v2 else _v1_header)(w, _dataset_msgs(pose, w, v2))
    if v2:
        grp = _link_group(w, headers, dense=dense_group)
        root_children = {group_name: grp}
        if extra_groups:
            root_children["poses"] = _link_group(w, {"0": pose_hdr})
        root = _link_group(w, root_children)
        eof = len(w.b)
        w.put(0, SIGNATURE + struct.pack("<BBBB", sbv, 8, 8, 0) + struct.pack("<QQQQ", 0, UNDEF, eof, root) + b"\0" * 4)
    else:
        grp, _, _ = _symbol_group(w, headers, leaf_k, internal_k)
        root_children = {group_name: grp}
        if extra_groups:
            root_children["poses"] = _symbol_group(w, {"0": pose_hdr}, leaf_k, internal_k)[0]
        root, rtree, rheap = _symbol_group(w, root_children, leaf_k, internal_k)
        eof = len(w.b)
        sb = SIGNATURE + struct.pack("<8B", sbv, 0, 0, 0, 0, 8, 8, 0) + struct.pack("<HHI", leaf_k, internal_k, 0)
        if sbv == 1:   # indexed storage internal node K, reserved
            sb += struct.pack("<HH", 32, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
        sb += struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", rtree, rheap)
        w.put(0, sb)
    data = bytes(w.b)
    if userblock:   # a user block before the superblock; addresses stay relative to it
        data = b"\0" * userblock + data
        base_field = {0: 24, 1: 28}.get(sbv, 12)
        data = bytearray(data)
        data[userblock + base_field:userblock + base_field + 8] = struct.pack("<Q", userblock)
        data = bytes(data)
    if v2:   # the superblock's checksum over its 44 bytes before it
        data = bytearray(data)
        data[userblock + 44:userblock + 48] = struct.pack("<I", lookup3(bytes(data[userblock:userblock + 44])))
        data = bytes(data)
    with open(path, "wb") as f:
        f.write(data)
