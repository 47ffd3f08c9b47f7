"""A second, independent reading of the HDF5 file-format specification, in
Python, for the tests of the library's Breakpoint%05d.h5 writer and reader
(hydrothermal3d_gb300/csrc/h5.cu):

* parse(path): walks a file the way the specification describes it
  (superblock version 0, root symbol table entry, local heap, group B-tree,
  symbol table node, version-1 object headers and their messages) and returns
  {name: (dims, float64 values)} plus the raw messages, checking every
  signature, version and size field on the way;
* build(datasets, ...): writes a file with structural choices the library's
  writer does not make (root group without a cached scratch-pad, compact
  storage, an object-header continuation block, dataspace version 2, extra
  messages the reader must skip), for the reader's tests.
"""
import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
F64LE = bytes([0x11, 0x20, 0x3F, 0x00, 8, 0, 0, 0, 0, 0, 64, 0, 52, 11, 0, 52, 0xFF, 0x03, 0, 0])


def u(b, off, n):
    return int.from_bytes(b[off:off + n], "little")


def parse(path):
    b = open(path, "rb").read()
    assert b[:8] == SIG
    assert b[8] == 0 and b[13] == 8 and b[14] == 8  # superblock v0, 8-byte offsets and lengths
    leaf_k, int_k = u(b, 16, 2), u(b, 18, 2)
    assert (leaf_k, int_k) == (4, 16)
    assert u(b, 24, 8) == 0 and u(b, 32, 8) == UNDEF and u(b, 48, 8) == UNDEF
    assert u(b, 40, 8) == len(b)  # end-of-file address
    root = 56
    assert u(b, root + 16, 4) == 1
    btree, heap = u(b, root + 24, 8), u(b, root + 32, 8)
    oh = u(b, root + 8, 8)
    msgs = object_header(b, oh)
    assert msgs == [(0x0011, struct.pack("<QQ", btree, heap))]
    assert b[heap:heap + 4] == b"HEAP" and b[heap + 4] == 0
    hsize, free, hdata = u(b, heap + 8, 8), u(b, heap + 16, 8), u(b, heap + 24, 8)
    assert free == 1  # no free block
    assert b[hdata] == 0  # offset 0: the empty name
    assert b[btree:btree + 4] == b"TREE" and b[btree + 4] == 0 and b[btree + 5] == 0
    used = u(b, btree + 6, 2)
    assert used == 1 and u(b, btree + 8, 8) == UNDEF and u(b, btree + 16, 8) == UNDEF
    key0, snod, key1 = u(b, btree + 24, 8), u(b, btree + 32, 8), u(b, btree + 40, 8)
    assert key0 == 0
    assert b[btree + 48:btree + 544] == bytes(496)  # unused keys and children of the 2K = 32 node
    assert b[snod:snod + 4] == b"SNOD" and b[snod + 4] == 1
    ns = u(b, snod + 6, 2)
    names, out = [], {}
    for e in range(ns):
        p = snod + 8 + 40 * e
        off, ohd, cache = u(b, p, 8), u(b, p + 8, 8), u(b, p + 16, 4)
        assert cache == 0 and off < hsize
        name = b[hdata + off:b.index(b"\0", hdata + off)].decode()
        names.append(name)
        m = dict(object_header(b, ohd))
        ds = m[0x0001]
        assert ds[0] == 1  # dataspace version 1
        rank = ds[1]
        dims = tuple(u(ds, 8 + 8 * a, 8) for a in range(rank))
        assert m[0x0003][:20] == F64LE
        lay = m[0x0008]
        assert lay[0] == 3 and lay[1] == 1  # layout version 3, contiguous
        addr, size = u(lay, 2, 8), u(lay, 10, 8)
        n = int(np.prod(dims)) if rank else 1
        assert size == 8 * n and addr + size <= len(b)
        out[name] = (dims, np.frombuffer(b[addr:addr + size], "<f8"))
    assert names == sorted(names, key=lambda s: s.encode())  # strcmp order
    assert key1 == next(o for o in range(hsize) if b[hdata + o:].startswith(names[-1].encode() + b"\0"))
    return out


def object_header(b, oh):
    """[(type, data)] of a version-1 object header (no continuation blocks)."""
    assert b[oh] == 1 and b[oh + 1] == 0
    n, refc, size = u(b, oh + 2, 2), u(b, oh + 4, 4), u(b, oh + 8, 4)
    assert refc == 1 and oh % 8 == 0
    res, p = [], oh + 16
    for _ in range(n):
        t, sz = u(b, p, 2), u(b, p + 2, 2)
        assert sz % 8 == 0
        res.append((t, b[p + 8:p + 8 + sz]))
        p += 8 + sz
    assert p == oh + 16 + size
    return res


# ------------------------------------------------------------------ builder
class _W:
    def __init__(self):
        self.b = bytearray()

    def at(self):
        return len(self.b)

    def put(self, data):
        a = len(self.b)
        self.b += data
        while len(self.b) % 8:
            self.b += b"\0"
        return a


def _msg(t, data):
    data = bytes(data) + bytes((-len(data)) % 8)
    return struct.pack("<HHB3x", t, len(data), 0) + data


def _oh(msgs):
    body = b"".join(msgs)
    return struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(body)) + body


def build(path, datasets, cache_root=False, compact_scalars=True, continuation=True, dataspace_v2=True,
          extra_messages=True):
    """datasets: {name: numpy float64 array (C order, HDF5 dims = array.shape) or float}."""
    w = _W()
    w.put(bytes(96))  # superblock, filled in at the end
    names = sorted(datasets, key=lambda s: s.encode())
    heap_data = b"\0" * 8
    offs = {}
    for nm in names:
        offs[nm] = len(heap_data)
        e = nm.encode() + b"\0"
        heap_data += e + bytes((-len(e)) % 8)
    # raw data first (anywhere in the file is allowed)
    addr = {}
    for nm in names:
        v = datasets[nm]
        if isinstance(v, np.ndarray):
            addr[nm] = w.put(np.ascontiguousarray(v, "<f8").tobytes())
    ohs = {}
    for nm in names:
        v = datasets[nm]
        if isinstance(v, np.ndarray):
            dims = v.shape
            if dataspace_v2:
                dsp = struct.pack("<BBBB", 2, len(dims), 0, 1) + b"".join(struct.pack("<Q", d) for d in dims)
            else:
                dsp = struct.pack("<BBBB4x", 1, len(dims), 0, 0) + b"".join(struct.pack("<Q", d) for d in dims)
            lay = struct.pack("<BBQQ", 3, 1, addr[nm], 8 * v.size)
        else:
            dsp = struct.pack("<BBBB", 2, 0, 0, 0) if dataspace_v2 else struct.pack("<BBBB4x", 1, 0, 0, 0)
            val = struct.pack("<d", float(v))
            if compact_scalars:
                lay = struct.pack("<BBH", 3, 0, 8) + val
            else:
                lay = struct.pack("<BBQQ", 3, 1, w.put(val), 8)
        first = [_msg(0x0001, dsp), _msg(0x0003, F64LE)]
        if extra_messages:
            first.append(_msg(0x0012, struct.pack("<B3xI", 1, 1700000000)))  # modification time
            first.append(_msg(0x0000, bytes(16)))  # NIL
        second = [_msg(0x0008, lay)]
        if continuation:
            cont_block = b"".join(second)
            ca = w.put(cont_block)
            first.append(_msg(0x0010, struct.pack("<QQ", ca, len(cont_block))))
            ohs[nm] = w.put(_oh_n(first, len(first) + len(second)))
        else:
            ohs[nm] = w.put(_oh(first + second))
    snod = w.put(b"SNOD" + struct.pack("<BBH", 1, 0, len(names)) + b"".join(
        struct.pack("<QQI4x16x", offs[nm], ohs[nm], 0) for nm in names) + bytes(40 * (8 - len(names))))
    heap_d = w.put(heap_data)
    heap = w.put(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), 1, heap_d))
    btree = w.put(b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, UNDEF, UNDEF) +
                  struct.pack("<QQQ", 0, snod, offs[names[-1]]) + bytes(544 - 48))
    root_oh = w.put(_oh([_msg(0x0011, struct.pack("<QQ", btree, heap))]))
    eof = len(w.b)
    sb = SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0) + struct.pack(
        "<QQQQ", 0, UNDEF, eof, UNDEF)
    if cache_root:
        sb += struct.pack("<QQI4xQQ", 0, root_oh, 1, btree, heap)
    else:
        sb += struct.pack("<QQI4x16x", 0, root_oh, 0)
    w.b[:96] = sb
    with open(path, "wb") as f:
        f.write(bytes(w.b))


def _oh_n(msgs, n_total):
    """Object header whose message count includes the messages of its continuation block."""
    body = b"".join(msgs)
    return struct.pack("<BBHII4x", 1, 0, n_total, 1, len(body)) + body
