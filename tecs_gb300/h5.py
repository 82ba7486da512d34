"""Minimal HDF5 reader and writer for cell snapshots (no libhdf5 needed).

The reference writes snapshots with HighFive/libhdf5 (include/io/hdf5_writer.hpp:
120-129 write_single, :306-321 write): one group "t<step>" per call holding one
dataset per field, named by the field's label ("position", "polarity", ...),
shaped [active_count, components], little-endian float32, plus an XDMF
sidecar.  libhdf5 is not available here, so this module writes and reads that
subset of the HDF5 file format itself, following the public format
specification (version 0 superblock, version 1 object headers, symbol-table
groups built from a version 1 B-tree, a symbol table node and a local heap,
contiguous datasets described by dataspace v1, datatype v1, fill value v2 and
layout v3 messages) and laid out the way the HDF5 library lays out the
reference's own fixture files (examples/data/sphere_ic.h5).

Writer: snapshots are appended as they arrive (data and the new group's
metadata at the end of the file; the root group's heap, symbol table nodes and
B-tree nodes are rewritten in place), so a running simulation streams into one
file.  The root group takes any number of groups: its B-tree gains levels
(32 children per node) as the symbol table nodes (8 entries each) grow, and
its name heap moves to a segment twice the size when it fills, as the HDF5
library does; the root node and the heap header stay where they are.
"""
from __future__ import annotations

import bisect
import os
import struct
import threading
from pathlib import Path
from typing import Dict, List, Optional, Tuple

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIG = b"\x89HDF\r\n\x1a\n"
LEAF_K = 4          # group leaf node K: a symbol table node holds 2K entries
INTERNAL_K = 16     # group internal node K: a B-tree node holds 2K children
SNOD_ENTRIES = 2 * LEAF_K
ENTRY_SIZE = 40
SNOD_SIZE = 8 + SNOD_ENTRIES * ENTRY_SIZE
BTREE_SIZE = 24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8
ROOT_HEAP_DATA = 8192


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ---------------------------------------------------------------------------
# messages

def _msg(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = body + b"\0" * (_pad8(len(body)) - len(body))
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _dataspace(shape: Tuple[int, ...]) -> bytes:
    body = struct.pack("<BBB5x", 1, len(shape), 1)
    body += b"".join(struct.pack("<Q", d) for d in shape)   # dimensions
    body += b"".join(struct.pack("<Q", d) for d in shape)   # maximum dimensions
    return _msg(0x0001, body)


def _datatype(dtype: np.dtype) -> bytes:
    dtype = np.dtype(dtype)
    if dtype == np.float32:
        # version 1, class 1 (floating point); little endian, IEEE layout
        body = bytes([0x11, 0x20, 0x1F, 0x00]) + struct.pack("<I", 4)
        body += struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
    elif dtype == np.float64:
        body = bytes([0x11, 0x20, 0x3F, 0x00]) + struct.pack("<I", 8)
        body += struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    elif dtype in (np.int32, np.uint32, np.int64, np.uint64):
        signed = 0x08 if dtype.kind == "i" else 0x00
        body = bytes([0x10, signed, 0x00, 0x00]) + struct.pack("<I", dtype.itemsize)
        body += struct.pack("<HH", 0, 8 * dtype.itemsize)
    else:
        raise TypeError(f"unsupported dtype {dtype}")
    return _msg(0x0003, body, flags=1)


def _fill_value() -> bytes:
    # version 2, allocation time late, fill written if set, defined with size 0
    # (the library's default, as in the reference's fixture files)
    return _msg(0x0005, struct.pack("<BBBBI", 2, 2, 2, 1, 0), flags=1)


def _layout_contiguous(addr: int, size: int) -> bytes:
    return _msg(0x0008, struct.pack("<BBQQ", 3, 1, addr, size))


def _symbol_table_msg(btree: int, heap: int) -> bytes:
    return _msg(0x0011, struct.pack("<QQ", btree, heap))


def _object_header(messages: List[bytes], min_size: int = 0) -> bytes:
    body = b"".join(messages)
    if len(body) < min_size:  # a NIL message pads the header like the library does
        pad = min_size - len(body)
        if pad < 8:
            pad += 8
        body += struct.pack("<HHB3x", 0, pad - 8, 0) + b"\0" * (pad - 8)
        n = len(messages) + 1
    else:
        n = len(messages)
    return struct.pack("<BBHII4x", 1, 0, n, 1, len(body)) + body


def _entry(name_off: int, ohdr: int, btree: Optional[int] = None, heap: Optional[int] = None) -> bytes:
    if btree is None:
        return struct.pack("<QQII16x", name_off, ohdr, 0, 0)
    return struct.pack("<QQIIQQ", name_off, ohdr, 1, 0, btree, heap)


def _snod(entries: List[bytes]) -> bytes:
    out = b"SNOD" + struct.pack("<BBH", 1, 0, len(entries)) + b"".join(entries)
    return out + b"\0" * (SNOD_SIZE - len(out))


def _btree(keys: List[int], children: List[int], level: int = 0, left: int = UNDEF, right: int = UNDEF) -> bytes:
    out = b"TREE" + struct.pack("<BBHQQ", 0, level, len(children), left, right)
    for k in range(len(children)):
        out += struct.pack("<QQ", keys[k], children[k])
    out += struct.pack("<Q", keys[len(children)])
    return out + b"\0" * (BTREE_SIZE - len(out))


def _heap_header(data_size: int, free_off: int, data_addr: int) -> bytes:
    return b"HEAP" + struct.pack("<B3xQQQ", 0, data_size, free_off, data_addr)


class _Heap:
    """Local heap data segment: NUL-terminated names, each padded to 8 bytes."""

    def __init__(self, size: int):
        self.size = size
        self.data = bytearray(8)  # offset 0: the empty name

    def fits(self, name: str) -> bool:
        return len(self.data) + _pad8(len(name.encode()) + 1) + 16 <= self.size

    def add(self, name: str) -> int:
        off = len(self.data)
        raw = name.encode() + b"\0"
        self.data += raw + b"\0" * (_pad8(len(raw)) - len(raw))
        if len(self.data) + 16 > self.size:
            raise ValueError("group name heap full")
        return off

    def segment(self, start: int = 0, full: bool = True) -> Tuple[bytes, int]:
        """(data bytes of the segment from `start`, free-list head offset); full=False stops after the free
        block's header (what changes when a name is added to a segment whose rest is zero)"""
        used = len(self.data)
        free = self.size - used
        out = bytes(self.data[start:])
        if free >= 16:
            out += struct.pack("<QQ", 1, free) + (b"\0" * (free - 16) if full else b"")  # one free block, last
            return out, used
        return out + b"\0" * free, UNDEF


# ---------------------------------------------------------------------------
# writer

class H5Writer:
    """Append-only HDF5 file of groups of float32 datasets (t<step>/<field>).

    append=True continues a file this writer made (closed, or left by a writer that stopped mid-run) with
    the state it had after its last complete group, so the file ends as if one writer had written every
    group; a missing or empty file is created."""

    def __init__(self, path: str | os.PathLike, append: bool = False):
        self.path = Path(path)
        resume = append and self.path.exists() and self.path.stat().st_size > 0
        self.f = open(self.path, "rb+" if resume else "wb+")
        self.names: Dict[str, Tuple[int, int, int, int]] = {}  # group name -> (name_off, ohdr, btree, heap)
        self.order: List[str] = []  # group names in name order
        self.heap = _Heap(ROOT_HEAP_DATA)
        # fixed metadata region: superblock, root object header, B-tree, heap header + data, first SNODs
        self.root_ohdr = 96                     # after the 96-byte superblock
        self.root_btree = self.root_ohdr + 40   # object header prefix + symbol table message
        self.root_heap = self.root_btree + BTREE_SIZE
        self.root_heap_data = self.root_heap + 32
        self.snods: List[int] = []
        self.nodes: List[List[int]] = []  # B-tree nodes below the root, per level (leaf level first)
        self.eof = self.root_heap_data + ROOT_HEAP_DATA
        if resume:
            self._load()
        else:
            self._write_root()

    def _load(self):
        """The writer's state from the root metadata of a file it wrote (the superblock, written last by
        every group write, holds the end of the last complete group)."""
        self.f.seek(0)
        b = self.f.read()
        if b[:8] != SIG or struct.unpack_from("<QII", b, 64) != (self.root_ohdr, 1, 0) or \
                struct.unpack_from("<QQ", b, 80) != (self.root_btree, self.root_heap):
            raise ValueError(f"{self.path} was not written by this writer")
        self.eof = struct.unpack_from("<Q", b, 40)[0]
        size, free, data = struct.unpack_from("<QQQ", b, self.root_heap + 8)
        self.heap = _Heap(size)
        self.heap.data = bytearray(b[data:data + (size if free == UNDEF else free)])
        self.root_heap_data = data

        def walk(node):
            _, level, used = struct.unpack_from("<BBH", b, node + 4)
            for k in range(used):
                child = struct.unpack_from("<Q", b, node + 32 + 16 * k)[0]
                if level:
                    while len(self.nodes) < level:
                        self.nodes.append([])
                    self.nodes[level - 1].append(child)
                    walk(child)
                else:
                    self.snods.append(child)

        walk(self.root_btree)
        for sn in self.snods:
            for e in range(struct.unpack_from("<H", b, sn + 6)[0]):
                name_off, ohdr, _, _, btree, heap = struct.unpack_from("<QQIIQQ", b, sn + 8 + ENTRY_SIZE * e)
                name = b[data + name_off:b.index(b"\0", data + name_off)].decode()
                self.names[name] = (name_off, ohdr, btree, heap)
                self.order.append(name)

    def _write_at(self, addr: int, data: bytes):
        self.f.seek(addr)
        self.f.write(data)

    def _alloc(self, size: int) -> int:
        addr = self.eof
        self.eof = _pad8(self.eof + size)
        return addr

    def _superblock(self) -> bytes:
        sb = SIG + struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0)
        sb += struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, self.eof, UNDEF)
        sb += _entry(0, self.root_ohdr, self.root_btree, self.root_heap)
        return sb

    def _write_root(self, first: int = 0, heap_from: int = 0):
        """Rewrite the root group's metadata; symbol table nodes before the one holding name-order entry
        `first`, and the name heap before offset `heap_from` (0: all of it), are unchanged and not
        rewritten."""
        n = len(self.order)
        nchunks = max(1, -(-n // SNOD_ENTRIES))
        while len(self.snods) < nchunks:
            self.snods.append(self._alloc(SNOD_SIZE))
        for k in range(first // SNOD_ENTRIES, nchunks):
            chunk = [_entry(*self.names[g]) for g in self.order[k * SNOD_ENTRIES:(k + 1) * SNOD_ENTRIES]]
            self._write_at(self.snods[k], _snod(chunk))
        # each child's largest name (heap offset); a node's keys: the bound left of its first child, then these
        children = self.snods[:nchunks]
        maxkey = [self.names[self.order[min(n, (k + 1) * SNOD_ENTRIES) - 1]][0] if n else 0 for k in range(nchunks)]
        level = 0
        while len(children) > 2 * INTERNAL_K:
            width = 2 * INTERNAL_K
            count = -(-len(children) // width)
            if len(self.nodes) <= level:
                self.nodes.append([])
            addrs = self.nodes[level]
            while len(addrs) < count:
                addrs.append(self._alloc(BTREE_SIZE))
            up = []
            for j in range(count):
                kids, keys = children[j * width:(j + 1) * width], maxkey[j * width:(j + 1) * width]
                left_key = maxkey[j * width - 1] if j else 0
                self._write_at(addrs[j], _btree([left_key] + keys, kids, level, addrs[j - 1] if j else UNDEF,
                                                addrs[j + 1] if j + 1 < count else UNDEF))
                up.append(keys[-1])
            children, maxkey = addrs[:count], up
            level += 1
        self._write_at(self.root_btree, _btree([0] + maxkey, children, level))
        seg, free = self.heap.segment(heap_from, full=heap_from == 0)
        self._write_at(self.root_heap, _heap_header(self.heap.size, free, self.root_heap_data))
        self._write_at(self.root_heap_data + heap_from, seg)
        self._write_at(self.root_ohdr, _object_header([_symbol_table_msg(self.root_btree, self.root_heap)]))
        self._write_at(0, self._superblock())

    def write_group(self, group: str, datasets: Dict[str, np.ndarray]):
        """One group of datasets, like HDF5_Writer::write for one step."""
        if group in self.names:
            raise ValueError(f"group {group} exists")
        if len(datasets) > SNOD_ENTRIES:
            raise ValueError("at most 8 datasets per group")
        # the group's own heap with the dataset names
        gheap = _Heap(_pad8(8 + sum(_pad8(len(k) + 1) for k in datasets) + 16))
        name_offs = {k: gheap.add(k) for k in datasets}
        ds_entries = []
        for name in sorted(datasets):
            arr = np.ascontiguousarray(datasets[name])
            if arr.dtype == np.float64:
                arr = arr.astype(np.float32)
            data_addr = self._alloc(max(arr.nbytes, 1))
            self._write_at(data_addr, arr.tobytes())
            ohdr = _object_header([_dataspace(arr.shape), _datatype(arr.dtype), _fill_value(),
                                   _layout_contiguous(data_addr if arr.nbytes else UNDEF, arr.nbytes)],
                                  min_size=216)
            oaddr = self._alloc(len(ohdr))
            self._write_at(oaddr, ohdr)
            ds_entries.append(_entry(name_offs[name], oaddr))
        snod = self._alloc(SNOD_SIZE)
        self._write_at(snod, _snod(ds_entries))
        btree = self._alloc(BTREE_SIZE)
        last = name_offs[sorted(datasets)[-1]] if datasets else 0
        self._write_at(btree, _btree([0, last], [snod]))
        seg, free = gheap.segment()
        heap = self._alloc(32)
        heap_data = self._alloc(len(seg))
        self._write_at(heap, _heap_header(len(seg), free, heap_data))
        self._write_at(heap_data, seg)
        gohdr = _object_header([_symbol_table_msg(btree, heap)], min_size=24)
        gaddr = self._alloc(len(gohdr))
        self._write_at(gaddr, gohdr)
        moved = not self.heap.fits(group)
        if moved:  # a segment twice the size at the end of the file
            while not self.heap.fits(group):
                self.heap.size *= 2
            self.root_heap_data = self._alloc(self.heap.size)
        name_off = self.heap.add(group)
        self.names[group] = (name_off, gaddr, btree, heap)
        at = bisect.bisect_left(self.order, group)
        self.order.insert(at, group)
        self._write_root(at, 0 if moved else name_off)
        self.f.flush()

    def close(self):
        if self.f:
            self._write_at(0, self._superblock())
            self.f.truncate(self.eof)
            self.f.close()
            self.f = None


# ---------------------------------------------------------------------------
# reader

class H5File:
    """Reads symbol-table groups and contiguous / compact datasets of fixed-size numeric types."""

    def __init__(self, path: str | os.PathLike):
        self.b = Path(path).read_bytes()
        if self.b[:8] != SIG:
            raise ValueError("not an HDF5 file")
        if self.b[8] != 0:
            raise ValueError(f"superblock version {self.b[8]} not supported")
        if self.b[13] != 8 or self.b[14] != 8:
            raise ValueError("only 8-byte offsets and lengths are supported")
        self.root = struct.unpack_from("<Q", self.b, 64)[0]

    def _messages(self, addr: int):
        b = self.b
        ver, _, nmsg, _, hsize = struct.unpack_from("<BBHII", b, addr)
        if ver != 1:
            raise ValueError(f"object header version {ver} not supported")
        blocks = [(addr + 16, hsize)]
        out = []
        while blocks:
            off, size = blocks.pop(0)
            end = off + size
            while off + 8 <= end:
                mtype, msize, _ = struct.unpack_from("<HHB", b, off)
                body = b[off + 8: off + 8 + msize]
                if mtype == 0x0010:
                    blocks.append(struct.unpack_from("<QQ", body, 0))
                else:
                    out.append((mtype, body))
                off += 8 + msize
        return out

    def _group_entries(self, ohdr: int) -> Dict[str, int]:
        msgs = dict(self._messages(ohdr))
        if 0x0011 not in msgs:
            raise ValueError("not a symbol-table group")
        btree, heap = struct.unpack_from("<QQ", msgs[0x0011], 0)
        b = self.b
        if b[heap:heap + 4] != b"HEAP":
            raise ValueError("bad local heap")
        _, _, data_addr = struct.unpack_from("<QQQ", b, heap + 8)
        out = {}

        def walk(node):
            if b[node:node + 4] != b"TREE":
                raise ValueError("bad B-tree node")
            ntype, level, nent = struct.unpack_from("<BBH", b, node + 4)
            for k in range(nent):
                child = struct.unpack_from("<Q", b, node + 24 + 16 * k + 8)[0]
                if level > 0:
                    walk(child)
                    continue
                if b[child:child + 4] != b"SNOD":
                    raise ValueError("bad symbol table node")
                nsym = struct.unpack_from("<H", b, child + 6)[0]
                for e in range(nsym):
                    name_off, oaddr = struct.unpack_from("<QQ", b, child + 8 + ENTRY_SIZE * e)
                    end = b.index(b"\0", data_addr + name_off)
                    out[b[data_addr + name_off:end].decode()] = oaddr

        walk(btree)
        return out

    def _resolve(self, path: str) -> int:
        addr = self.root
        for part in [p for p in path.strip("/").split("/") if p]:
            entries = self._group_entries(addr)
            if part not in entries:
                raise KeyError(path)
            addr = entries[part]
        return addr

    def keys(self, path: str = "/") -> List[str]:
        return sorted(self._group_entries(self._resolve(path)))

    @staticmethod
    def _shape(msgs) -> Tuple[int, ...]:
        ds = msgs[0x0001]
        ver, rank = ds[0], ds[1]
        off = 8 if ver == 1 else 4
        return tuple(struct.unpack_from("<Q", ds, off + 8 * k)[0] for k in range(rank))

    def shape(self, path: str) -> Tuple[int, ...]:
        return self._shape(dict(self._messages(self._resolve(path))))

    def read(self, path: str) -> np.ndarray:
        msgs = dict(self._messages(self._resolve(path)))
        shape = self._shape(msgs)
        dt = msgs[0x0003]
        cls = dt[0] & 0x0F
        size = struct.unpack_from("<I", dt, 4)[0]
        if dt[1] & 0x01:
            raise ValueError("big-endian data not supported")
        if cls == 1:
            dtype = {4: np.float32, 8: np.float64}[size]
        elif cls == 0:
            dtype = np.dtype(("i" if dt[1] & 0x08 else "u") + str(size))
        else:
            raise ValueError(f"datatype class {cls} not supported")
        lay = msgs[0x0008]
        if lay[0] != 3:
            raise ValueError("only layout message version 3 is supported")
        count = int(np.prod(shape)) if shape else 1
        if lay[1] == 1:  # contiguous
            addr, nbytes = struct.unpack_from("<QQ", lay, 2)
            if addr == UNDEF:
                return np.zeros(shape, dtype)
            raw = self.b[addr:addr + nbytes]
        elif lay[1] == 0:  # compact
            nbytes = struct.unpack_from("<H", lay, 2)[0]
            raw = lay[4:4 + nbytes]
        else:
            raise ValueError("chunked datasets are not supported")
        return np.frombuffer(raw, dtype=dtype, count=count).reshape(shape).copy()


# ---------------------------------------------------------------------------
# XDMF sidecar

class XdmfSidecar:
    """The XDMF sidecar "<path>.xmf" of the snapshot file "<path>.h5", for visualisation tools, in the
    reference writer's text (include/io/hdf5_writer.hpp:134-287): one temporal collection; per write a
    uniform grid whose geometry is the first field, the others node attributes ("Scalar" for one column,
    "Vector" for 2 or 3, "Tensor" for 9, else "Matrix"), a links field the grid's polyline topology in
    place of the cells as vertices; the static fields in every later grid.  Text is kept until it passes
    `threshold` characters, then appended to the file; close() ends the document."""

    def __init__(self, path: str | os.PathLike, threshold: int = 65536):
        path = Path(path)
        self.file = path.name + ".h5"
        self.f = open(str(path) + ".xmf", "w", newline="\n")
        self.threshold = threshold
        self.buf = ('<?xml version="1.0"?>\n<Xdmf Version="3.0">\n\t<Domain>\n'
                    '\t\t<Grid Name="Agents" GridType="Collection" CollectionType="Temporal">\n')
        self.static = ""

    def _item(self, group: str, label: str, arr: np.ndarray, link: bool = False) -> str:
        if len(arr) == 0:
            return ""
        cols = arr.shape[1] if arr.ndim > 1 else 0
        dims = f"{len(arr)} " + (f"{cols} " if cols else "")
        kind = "Scalar" if not cols else "Vector" if cols in (2, 3) else "Tensor" if cols == 9 else "Matrix"
        if link:
            out = (f'\t\t\t\t<Topology TopologyType="Polyline" NumberOfElements="{len(arr)}">\n'
                   '\t\t\t\t\t<DataItem Format="HDF" DataType="UInt32"')
        else:
            out = (f'\t\t\t\t<Attribute Name="{label}" AttributeType="{kind}" Center="Node">\n'
                   '\t\t\t\t\t<DataItem Format="HDF"')
        out += f' Dimensions="{dims}">\n\t\t\t\t\t\t{self.file}:{group}/{label}\n\t\t\t\t\t</DataItem>\n'
        return out + ("\t\t\t\t</Topology>\n" if link else "\t\t\t\t</Attribute>\n")

    def write(self, time: float, group: str, fields: List[Tuple[str, np.ndarray]], links: Tuple[str, ...] = ()):
        """One grid: `fields` in write order, the first the geometry; names in `links` are link fields."""
        (glabel, geom), rest = fields[0], fields[1:]
        n, d = len(geom), geom.shape[1]
        has_links = any(label in links and len(a) for label, a in rest)
        b = f'\t\t\t<Grid Name="{group}" GridType="Uniform">\n\t\t\t\t<Time Value="{time:f}'
        if not has_links:
            b += f'"/>\n\t\t\t\t<Topology TopologyType="Polyvertex" NumberOfElements="{n}'
        b += f'"/>\n\t\t\t\t<Geometry GeometryType="{"X" if d == 1 else "XY" if d == 2 else "XYZ"}">\n'
        b += f'\t\t\t\t\t<DataItem Format="HDF" Dimensions="{n} {d}">\n\t\t\t\t\t\t{self.file}:{group}/{glabel}\n'
        b += "\t\t\t\t\t</DataItem>\n\t\t\t\t</Geometry>\n"
        for label, a in rest:
            b += self._item(group, label, a, label in links)
        self.buf += b + self.static + "\t\t\t</Grid>\n"
        if len(self.buf) > self.threshold:
            self.f.write(self.buf)
            self.f.flush()
            self.buf = ""

    def write_static(self, fields: List[Tuple[str, np.ndarray]]):
        for label, a in fields:
            self.static += self._item("static", label, a)

    def close(self):
        if self.f:
            self.f.write(self.buf + "\t\t</Grid>\n\t</Domain>\n</Xdmf>\n")
            self.f.close()
            self.f = None


# ---------------------------------------------------------------------------
# snapshot sink used by the served loop

class SnapshotSink:
    """One HDF5 file per request, request_<index>.h5, one t<step> group per snapshot (position, polarity).
    With dt (the step's time) it also writes each file's XDMF sidecar, request_<index>.xmf, with time
    step * dt per grid.  append=True (a server resuming requests from their snapshots) continues existing
    files instead of starting them afresh, and their sidecars list the earlier snapshots too."""

    def __init__(self, directory: str | os.PathLike, dt: Optional[float] = None, append: bool = False):
        self.dir = Path(directory)
        self.dir.mkdir(parents=True, exist_ok=True)
        self.dt = dt
        self.append = append
        self.files: Dict[int, H5Writer] = {}
        self.sidecars: Dict[int, XdmfSidecar] = {}
        self.lock = threading.Lock()

    def __call__(self, request: int, step: int, positions: np.ndarray, polarity: Optional[np.ndarray]):
        with self.lock:
            w = self.files.get(request)
            if w is None:
                base = self.dir / f"request_{request:05d}"
                w = self.files[request] = H5Writer(str(base) + ".h5", append=self.append)
                if self.dt is not None:
                    x = self.sidecars[request] = XdmfSidecar(base)
                    if w.order:  # a continued file: its earlier snapshots' grids first, in step order
                        f = H5File(str(base) + ".h5")
                        for g in sorted(w.order, key=lambda g: int(g[1:])):
                            names = [nm for nm in ("position", "polarity") if nm in f.keys(g)]
                            x.write(int(g[1:]) * self.dt, g, [(nm, np.empty(f.shape(f"{g}/{nm}"), np.float32))
                                                             for nm in names])
            x = self.sidecars.get(request)
        fields = [("position", positions)] + ([("polarity", polarity)] if polarity is not None else [])
        w.write_group(f"t{step}", dict(fields))
        if x is not None:
            x.write(step * self.dt, f"t{step}", fields)

    def close(self):
        with self.lock:
            for w in self.files.values():
                w.close()
            for x in self.sidecars.values():
                x.close()
            self.files.clear()
            self.sidecars.clear()


def last_snapshot(directory: str | os.PathLike, request: int):
    """(step, positions, polarity or None) of the newest snapshot SnapshotSink wrote for a request, or None.

    A file whose writer stopped mid-run (a server that never closed it) holds
    every group written before the stop: each write rewrites and flushes the
    root metadata after the group's data.  A file with no group, or that does
    not parse, gives None."""
    path = Path(directory) / f"request_{request:05d}.h5"
    if not path.exists():
        return None
    try:
        f = H5File(path)
        steps = sorted(int(k[1:]) for k in f.keys() if k.startswith("t") and k[1:].isdigit())
    except Exception:
        return None
    if not steps:
        return None
    g = f"t{steps[-1]}"
    pos = f.read(f"{g}/position")
    try:
        pol = f.read(f"{g}/polarity")
    except Exception:
        pol = None
    return steps[-1], pos, pol
