"""A dependency-free reader and writer for the part of the HDF5 file format that
cardiax/io.py:13-110 uses through h5py: groups, and fixed-shape datasets of IEEE floats and
two's-complement integers (scalars included) stored contiguously.

The layout written is the one the HDF5 library produces with its default ("earliest") format
settings, as described by the HDF5 File Format Specification (version 2.0 of the document,
format objects of the 1.8 library):

* superblock version 0 at offset 0 (8-byte offsets and lengths, group leaf K 4, internal K 16),
  whose root symbol-table entry caches the root group's B-tree and heap addresses;
* version-1 object headers (16-byte prefix, messages aligned on 8 bytes);
* groups as symbol tables: a symbol-table message pointing at a version-1 group B-tree (one leaf
  level, keys are heap offsets of the largest name of the child to their left) whose children
  are symbol-table nodes (``SNOD``, up to 8 entries each, sorted by name) and a local heap
  (``HEAP``) holding the names;
* datasets with a version-1 dataspace (with maximum dimensions equal to the dimensions), a
  version-1 datatype, a version-2 fill-value message (allocation late, fill written if set,
  library default fill) and a version-3 contiguous data-layout message.

Raw data is placed as datasets are created, so ``dset[i] = x`` writes straight into the file;
the metadata is written when the file is closed.  Reading follows the same structures and
also accepts continuation chunks, compact layouts and big-endian types; anything else (chunked
storage, superblock versions 2-3, version-2 object headers) raises ``NotImplementedError``.
"""
from __future__ import annotations

import os
import struct
from typing import Dict, Iterator, Optional, Tuple, Union

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"
LEAF_K = 4          # group leaf node K: a symbol-table node holds 2K entries
INTERNAL_K = 16     # group internal node K: a B-tree node has room for 2K children
SUPERBLOCK_SIZE = 96
ENTRY_SIZE = 40     # symbol-table entry with 8-byte offsets
SNOD_SIZE = 8 + 2 * LEAF_K * ENTRY_SIZE
BTREE_SIZE = 24 + 2 * INTERNAL_K * 8 + (2 * INTERNAL_K + 1) * 8
HEAP_FREE_NULL = 1  # "no next free block" in a local heap free list

# header message types
MSG_NIL, MSG_DATASPACE, MSG_DATATYPE, MSG_FILL_OLD, MSG_FILL = 0x0, 0x1, 0x3, 0x4, 0x5
MSG_LAYOUT, MSG_CONTINUATION, MSG_SYMBOL_TABLE = 0x8, 0x10, 0x11


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ---------------------------------------------------------------------------------- datatypes

def _encode_datatype(dt: np.dtype) -> bytes:
    """Datatype message body (version 1) for a little-endian float or integer dtype."""
    dt = np.dtype(dt)
    if dt.byteorder == ">":
        raise ValueError("only little-endian data is written")
    if dt.kind == "f" and dt.itemsize in (4, 8):
        if dt.itemsize == 4:
            sign, exp_loc, exp_size, mant_size, bias = 31, 23, 8, 23, 127
        else:
            sign, exp_loc, exp_size, mant_size, bias = 63, 52, 11, 52, 1023
        head = bytes([0x10 | 1, 0x20, sign, 0]) + struct.pack("<I", dt.itemsize)
        props = struct.pack("<HHBBBBI", 0, 8 * dt.itemsize, exp_loc, exp_size, 0, mant_size,
                            bias)
        return head + props
    if dt.kind in "iu":
        flags = 0x08 if dt.kind == "i" else 0x00
        head = bytes([0x10 | 0, flags, 0, 0]) + struct.pack("<I", dt.itemsize)
        return head + struct.pack("<HH", 0, 8 * dt.itemsize)
    raise TypeError(f"datatype {dt} is not supported (IEEE float or integer only)")


def _decode_datatype(body: bytes) -> np.dtype:
    cls, version = body[0] & 0x0F, body[0] >> 4
    bits = body[1] | (body[2] << 8) | (body[3] << 16)
    size = struct.unpack_from("<I", body, 4)[0]
    order = ">" if bits & 1 else "<"
    if version not in (1, 2, 3):
        raise NotImplementedError(f"datatype message version {version}")
    if cls == 1 and size in (2, 4, 8):
        return np.dtype(f"{order}f{size}")
    if cls == 0 and size in (1, 2, 4, 8):
        return np.dtype(f"{order}{'i' if bits & 0x08 else 'u'}{size}")
    raise NotImplementedError(f"datatype class {cls} of size {size}")


# ------------------------------------------------------------------------------------ objects

class Dataset:
    """A fixed-shape dataset; ``d[key]`` reads and ``d[key] = value`` writes like an ndarray."""

    def __init__(self, file: "File", name: str, shape: Tuple[int, ...], dtype: np.dtype,
                 addr: int, layout: str = "contiguous", compact: bytes = b""):
        self.file, self.name = file, name
        self.shape, self.dtype = tuple(int(s) for s in shape), np.dtype(dtype)
        self.addr, self._layout, self._compact = addr, layout, compact

    @property
    def size(self) -> int:
        return int(np.prod(self.shape, dtype=np.int64))

    @property
    def nbytes(self) -> int:
        return self.size * self.dtype.itemsize

    @property
    def ndim(self) -> int:
        return len(self.shape)

    def __len__(self) -> int:
        if not self.shape:
            raise TypeError("a scalar dataset has no length")
        return self.shape[0]

    def _view(self, writable: bool) -> np.ndarray:
        if self._layout == "compact":
            a = np.frombuffer(self._compact, self.dtype, count=self.size).reshape(self.shape)
            return a.copy() if writable else a
        if self.nbytes == 0 or self.addr == UNDEF:
            if writable and self.nbytes:
                raise OSError(f"dataset {self.name} has no storage")
            return np.zeros(self.shape, self.dtype)
        if self.nbytes <= (1 << 16) and not writable:
            raw = self.file._read(self.addr, self.nbytes)
            return np.frombuffer(raw, self.dtype).reshape(self.shape)
        self.file._flush()
        mode = "r+" if writable else "r"
        return np.memmap(self.file.filename, dtype=self.dtype, mode=mode, offset=self.addr,
                         shape=self.shape if self.shape else (1,)).reshape(self.shape)

    def __getitem__(self, key) -> Union[np.ndarray, np.generic]:
        out = self._view(False)[key]
        return np.array(out) if isinstance(out, np.ndarray) else out

    def __setitem__(self, key, value):
        if self.file.mode == "r":
            raise OSError("file is open read-only")
        if self._layout != "contiguous":
            raise NotImplementedError("writing is supported for contiguous datasets only")
        m = self._view(True)
        m[key] = np.asarray(value, dtype=self.dtype)
        if isinstance(m, np.memmap):
            m.flush()
        del m

    def __array__(self, dtype=None, copy=None):
        a = self[()]
        return np.asarray(a, dtype=dtype)

    def __repr__(self) -> str:
        return f'<HDF5 dataset "{self.name}": shape {self.shape}, type "{self.dtype.str}">'


class Group:
    """A group: a mapping from names to datasets and groups, in name order."""

    def __init__(self, file: "File", name: str):
        self.file, self.name = file, name
        self._members: Dict[str, Union["Group", Dataset]] = {}

    # lookup ------------------------------------------------------------------------------------
    def _resolve(self, path: str):
        node: Union[Group, Dataset] = self.file if path.startswith("/") else self
        for p in (p for p in path.split("/") if p):
            if not isinstance(node, Group):
                raise KeyError(f"{path}: {node.name} is not a group")
            if p not in node._members:
                raise KeyError(f"unable to open object '{path}' (not found)")
            node = node._members[p]
        return node

    def __getitem__(self, key) -> Union["Group", Dataset]:
        if not isinstance(key, (str, bytes)):
            raise TypeError(f"Accessing a group is done with bytes or str, not {type(key)}")
        return self._resolve(key.decode() if isinstance(key, bytes) else key)

    def __contains__(self, key) -> bool:
        try:
            self._resolve(key)
            return True
        except KeyError:
            return False

    def __iter__(self) -> Iterator[str]:
        return iter(sorted(self._members, key=lambda s: s.encode()))

    def __len__(self) -> int:
        return len(self._members)

    def keys(self):
        return list(iter(self))

    def values(self):
        return [self._members[k] for k in self]

    def items(self):
        return [(k, self._members[k]) for k in self]

    # creation ----------------------------------------------------------------------------------
    def _parent(self, name: str) -> Tuple["Group", str]:
        """The group that will hold ``name`` (intermediate groups created) and the leaf name."""
        self.file._check_writable()
        parts = [p for p in name.split("/") if p]
        if not parts:
            raise ValueError("empty name")
        node: Union[Group, Dataset] = self.file if name.startswith("/") else self
        for p in parts[:-1]:
            if p not in node._members:
                node._members[p] = Group(self.file, _join(node.name, p))
            node = node._members[p]
            if not isinstance(node, Group):
                raise KeyError(f"{node.name} is not a group")
        if parts[-1] in node._members:
            raise ValueError(f"unable to create '{name}' (name already exists)")
        return node, parts[-1]

    def create_group(self, name: str) -> "Group":
        parent, leaf = self._parent(name)
        g = Group(self.file, _join(parent.name, leaf))
        parent._members[leaf] = g
        return g

    def require_group(self, name: str) -> "Group":
        return self[name] if name in self else self.create_group(name)

    def create_dataset(self, name: str, shape=None, dtype=None, data=None) -> Dataset:
        """A new dataset (``shape``/``dtype``, zero-filled, or ``data``), its storage allocated
        at once.  Python floats become float64, Python ints int64, as h5py stores them."""
        if data is not None:
            arr = np.asarray(data)
            if arr.dtype == np.float16 or arr.dtype.kind not in "fiu":
                raise TypeError(f"datatype {arr.dtype} is not supported")
            if dtype is not None:
                arr = arr.astype(dtype)
            if shape is not None and tuple(shape) != arr.shape:
                arr = arr.reshape(shape)
            shape, dtype = arr.shape, arr.dtype.newbyteorder("<")
        else:
            if shape is None:
                raise TypeError("one of shape or data must be given")
            shape = (int(shape),) if np.isscalar(shape) else tuple(int(s) for s in shape)
            dtype = np.dtype(dtype if dtype is not None else "f4").newbyteorder("<")
            _encode_datatype(dtype)  # reject unsupported types before allocating
        parent, leaf = self._parent(name)
        nbytes = int(np.prod(shape, dtype=np.int64)) * np.dtype(dtype).itemsize
        addr = self.file._allocate(nbytes) if nbytes else UNDEF
        d = Dataset(self.file, _join(parent.name, leaf), shape, dtype, addr)
        parent._members[leaf] = d
        if data is not None and nbytes:
            self.file._write(addr, np.ascontiguousarray(arr, dtype=d.dtype).tobytes())
        return d

    def __repr__(self) -> str:
        return f'<HDF5 group "{self.name}" ({len(self)} members)>'


def _join(parent: str, leaf: str) -> str:
    return ("/" + leaf) if parent in ("", "/") else parent + "/" + leaf


class File(Group):
    """``File(path, "w")`` creates (truncates) a file, ``File(path)`` / ``"r"`` opens one for
    reading, ``"r+"`` for reading and writing dataset contents in place."""

    def __init__(self, path: Union[str, os.PathLike], mode: str = "r"):
        if mode not in ("r", "r+", "w"):
            raise ValueError(f"mode {mode!r} is not supported (r, r+ or w)")
        self.filename, self.mode = os.fspath(path), mode
        Group.__init__(self, self, "/")
        self._closed = False
        if mode == "w":
            self._fh = open(self.filename, "w+b", buffering=0)
            self._eof = SUPERBLOCK_SIZE
            self._fh.truncate(self._eof)
        else:
            self._fh = open(self.filename, "rb" if mode == "r" else "r+b", buffering=0)
            self._eof = os.fstat(self._fh.fileno()).st_size
            _Reader(self).read_root()

    # raw access ----------------------------------------------------------------------------------
    def _check_writable(self):
        if self.mode != "w":
            raise OSError("objects can be created only in a file opened with mode 'w'")

    def _allocate(self, nbytes: int) -> int:
        addr = self._eof
        self._eof = addr + _pad8(nbytes)
        self._fh.truncate(self._eof)  # the new storage reads as zeros
        return addr

    def _write(self, addr: int, data: bytes):
        self._fh.seek(addr)
        self._fh.write(data)

    def _read(self, addr: int, n: int) -> bytes:
        self._fh.seek(addr)
        b = self._fh.read(n)
        if len(b) != n:
            raise OSError(f"truncated file: {n} bytes at {addr} past the end")
        return b

    def _flush(self):
        self._fh.flush()

    # lifetime ------------------------------------------------------------------------------------
    def close(self):
        if self._closed:
            return
        try:
            if self.mode == "w":
                _Writer(self).write()
            self._fh.flush()
        finally:
            self._fh.close()
            self._closed = True

    def flush(self):
        self._fh.flush()

    def __enter__(self) -> "File":
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __repr__(self) -> str:
        return f'<HDF5 file "{os.path.basename(self.filename)}" (mode {self.mode})>'


# ------------------------------------------------------------------------------------- writing

def _message(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = body + b"\0" * (_pad8(len(body)) - len(body))
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _object_header(messages) -> bytes:
    chunk = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(chunk)) + chunk


def _entry(name_offset: int, header: int, scratch: Optional[Tuple[int, int]] = None) -> bytes:
    if scratch is None:
        return struct.pack("<QQII16x", name_offset, header, 0, 0)
    return struct.pack("<QQIIQQ", name_offset, header, 1, 0, scratch[0], scratch[1])


class _Writer:
    def __init__(self, f: File):
        self.f = f

    def _put(self, data: bytes) -> int:
        addr = self.f._eof
        self.f._eof = addr + _pad8(len(data))
        self.f._write(addr, data + b"\0" * (_pad8(len(data)) - len(data)))
        return addr

    def _dataset_header(self, d: Dataset) -> int:
        rank = len(d.shape)
        space = struct.pack("<BBBB4x", 1, rank, 1 if rank else 0, 0)
        if rank:
            space += struct.pack(f"<{rank}Q", *d.shape) + struct.pack(f"<{rank}Q", *d.shape)
        fill = struct.pack("<BBBBI", 2, 2, 2, 1, 0)
        layout = struct.pack("<BBQQ", 3, 1, d.addr, d.nbytes)
        return self._put(_object_header([
            _message(MSG_DATASPACE, space),
            _message(MSG_DATATYPE, _encode_datatype(d.dtype), flags=1),
            _message(MSG_FILL, fill, flags=1),
            _message(MSG_LAYOUT, layout),
        ]))

    def _group(self, g: Group) -> Tuple[int, int, int]:
        """Writes a group's members, then its heap, nodes and header: (header, btree, heap)."""
        names = sorted(g._members, key=lambda s: s.encode())
        if len(names) > 2 * LEAF_K * 2 * INTERNAL_K:
            raise ValueError(f"group {g.name} has more than {4 * LEAF_K * INTERNAL_K} members")
        entries = []
        for n in names:
            m = g._members[n]
            if isinstance(m, Group):
                entries.append((n, *self._group(m)))
            else:
                entries.append((n, self._dataset_header(m), None, None))
        # local heap: the empty name at offset 0, then each name NUL-terminated, 8-aligned
        heap = bytearray(b"\0" * 8)
        offsets = {}
        for n in names:
            offsets[n] = len(heap)
            b = n.encode() + b"\0"
            heap += b + b"\0" * (_pad8(len(b)) - len(b))
        heap_data = self._put(bytes(heap))
        heap_addr = self._put(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), HEAP_FREE_NULL,
                                                    heap_data))
        # symbol-table nodes of at most 2K entries each
        children, keys = [], [0]
        step = 2 * LEAF_K
        for i in range(0, len(entries), step):
            chunk = entries[i:i + step]
            body = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, len(chunk)))
            for n, hdr, bt, hp in chunk:
                body += _entry(offsets[n], hdr, None if bt is None else (bt, hp))
            body += b"\0" * (SNOD_SIZE - len(body))
            children.append(self._put(bytes(body)))
            keys.append(offsets[chunk[-1][0]])
        node = bytearray(b"TREE" + struct.pack("<BBHQQ", 0, 0, len(children), UNDEF, UNDEF))
        for k, c in zip(keys, children):  # key i, child i, ..., then the last key
            node += struct.pack("<QQ", k, c)
        node += struct.pack("<Q", keys[-1])
        node += b"\0" * (BTREE_SIZE - len(node))
        btree = self._put(bytes(node))
        header = self._put(_object_header([
            _message(MSG_SYMBOL_TABLE, struct.pack("<QQ", btree, heap_addr))]))
        return header, btree, heap_addr

    def write(self):
        f = self.f
        header, btree, heap = self._group(f)
        sb = bytearray(SIGNATURE)
        sb += bytes([0, 0, 0, 0, 0, 8, 8, 0])
        sb += struct.pack("<HHI", LEAF_K, INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, f._eof, UNDEF)
        sb += _entry(0, header, (btree, heap))
        assert len(sb) == SUPERBLOCK_SIZE
        f._write(0, bytes(sb))
        f._fh.truncate(f._eof)


# ------------------------------------------------------------------------------------- reading

class _Reader:
    def __init__(self, f: File):
        self.f = f

    def read_root(self):
        f = self.f
        sb = f._read(0, SUPERBLOCK_SIZE)
        if sb[:8] != SIGNATURE:
            raise OSError(f"{f.filename} is not an HDF5 file (no signature at offset 0)")
        version = sb[8]
        if version not in (0, 1):
            raise NotImplementedError(f"superblock version {version}")
        so, sl = sb[13], sb[14]
        if so != 8 or sl != 8:
            raise NotImplementedError(f"offset/length sizes {so}/{sl}")
        pos = 24 + (4 if version == 1 else 0)
        base, _, eof, _ = struct.unpack_from("<QQQQ", sb if version == 0 else
                                             f._read(0, SUPERBLOCK_SIZE + 4), pos)
        if base != 0:
            raise NotImplementedError("a non-zero base address")
        if eof > f._eof:
            raise OSError(f"truncated file: end of file address {eof}, size {f._eof}")
        raw = f._read(pos + 32, ENTRY_SIZE)
        _, header = struct.unpack_from("<QQ", raw, 0)
        self._fill_group(f, header)

    def _messages(self, addr: int):
        f = self.f
        pre = f._read(addr, 16)
        version, _, nmsg, _, size = struct.unpack_from("<BBHII", pre, 0)
        if pre[:4] == b"OHDR":
            raise NotImplementedError("version-2 object headers")
        if version != 1:
            raise OSError(f"object header at {addr}: version {version}")
        chunks, out = [(addr + 16, size)], []
        while chunks:
            start, length = chunks.pop(0)
            data = f._read(start, length)
            p = 0
            while p + 8 <= length and len(out) < nmsg:
                mtype, msize, flags = struct.unpack_from("<HHB", data, p)
                body = data[p + 8:p + 8 + msize]
                p += 8 + msize
                if mtype == MSG_CONTINUATION:
                    chunks.append(struct.unpack_from("<QQ", body, 0))
                out.append((mtype, flags, body))
        return out

    def _fill_group(self, g: Group, header: int):
        stab = [b for t, _, b in self._messages(header) if t == MSG_SYMBOL_TABLE]
        if not stab:
            raise NotImplementedError(f"group {g.name}: not a symbol-table group")
        btree, heap = struct.unpack_from("<QQ", stab[0], 0)
        hh = self.f._read(heap, 32)
        if hh[:4] != b"HEAP":
            raise OSError(f"group {g.name}: bad local heap signature")
        heap_size, _, heap_data = struct.unpack_from("<QQQ", hh, 8)
        names = self.f._read(heap_data, heap_size)
        for off, hdr, cache in self._btree_entries(btree):
            end = names.index(b"\0", off)
            name = names[off:end].decode()
            if any(t == MSG_SYMBOL_TABLE for t, _, _ in self._messages(hdr)):
                sub = Group(self.f, _join(g.name, name))
                self._fill_group(sub, hdr)
                g._members[name] = sub
            else:
                g._members[name] = self._dataset(_join(g.name, name), hdr)

    def _btree_entries(self, addr: int):
        f = self.f
        head = f._read(addr, 24)
        if head[:4] != b"TREE":
            raise OSError(f"bad B-tree signature at {addr}")
        ntype, level, used = struct.unpack_from("<BBH", head, 4)
        if ntype != 0:
            raise OSError("not a group B-tree")
        body = f._read(addr + 24, used * 16 + 8)
        children = [struct.unpack_from("<Q", body, 8 + 16 * i)[0] for i in range(used)]
        for c in children:
            if level > 0:
                yield from self._btree_entries(c)
                continue
            node = f._read(c, 8)
            if node[:4] != b"SNOD":
                raise OSError(f"bad symbol-table node signature at {c}")
            nsym = struct.unpack_from("<H", node, 6)[0]
            raw = f._read(c + 8, nsym * ENTRY_SIZE)
            for i in range(nsym):
                off, hdr, cache = struct.unpack_from("<QQI", raw, i * ENTRY_SIZE)
                yield off, hdr, cache

    def _dataset(self, name: str, header: int) -> Dataset:
        shape = dtype = None
        addr, layout, compact = UNDEF, None, b""
        for t, _, b in self._messages(header):
            if t == MSG_DATASPACE:
                version, rank, flags = b[0], b[1], b[2]
                if version == 1:
                    p = 8
                elif version == 2:
                    p = 4
                    if b[3] == 2:  # null dataspace
                        rank = 0
                else:
                    raise NotImplementedError(f"dataspace version {version}")
                shape = struct.unpack_from(f"<{rank}Q", b, p) if rank else ()
            elif t == MSG_DATATYPE:
                dtype = _decode_datatype(b)
            elif t == MSG_LAYOUT:
                if b[0] != 3:
                    raise NotImplementedError(f"data layout version {b[0]}")
                if b[1] == 1:
                    layout = "contiguous"
                    addr = struct.unpack_from("<Q", b, 2)[0]
                elif b[1] == 0:
                    layout = "compact"
                    n = struct.unpack_from("<H", b, 2)[0]
                    compact = bytes(b[4:4 + n])
                else:
                    raise NotImplementedError(f"dataset {name}: chunked or virtual storage")
        if shape is None or dtype is None or layout is None:
            raise OSError(f"dataset {name}: missing dataspace, datatype or layout")
        return Dataset(self.f, name, shape, dtype, addr, layout, compact)
