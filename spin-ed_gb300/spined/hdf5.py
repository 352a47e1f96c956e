"""Minimal HDF5 reader and writer for SpinED's result files.

SpinED writes its results through the HDF5 library (src/SpinED.hs:267-294,
315-337,354-368): groups /basis, /hamiltonian, /observables, /_workspace and
datasets /basis/representatives (uint64), /hamiltonian/eigenvalues,
/hamiltonian/eigenvectors, /hamiltonian/residuals and one dataset of
expectation values per observable. No HDF5 library is available to this
package, so this module implements the part of the HDF5 file format
(specification version 2 of the format document, "earliest" layout that the
HDF5 library itself writes by default) that those files need:

* superblock version 0 with 8-byte offsets and lengths;
* groups as version-1 object headers holding a symbol-table message, a
  version-1 B-tree (group nodes, K = 16) over symbol-table nodes (leaf K = 4)
  and a local heap of link names;
* datasets as version-1 object headers with a version-1 dataspace, a
  datatype (little-endian fixed-point, IEEE float, or the compound {r, i}
  that h5py also uses for complex numbers), a version-2 fill-value message
  and a version-3 contiguous layout;
* the reader also follows object-header continuation messages, multi-level
  group B-trees and compact layouts, and skips messages it does not use.

Files are rewritten whole (the tree is read, modified and written again),
which gives the reference's append/overwrite semantics (SpinED.hs:267-294,
354-360) for result files of the sizes exact diagonalisation produces.
"""
from __future__ import annotations

import os
import struct

import numpy as np

__all__ = ["Group", "read", "write", "H5Error"]

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"
GROUP_LEAF_K = 4
GROUP_INTERNAL_K = 16
FREE_NULL = 1  # end of a local heap's free list on disk


class H5Error(ValueError):
    pass


class Group(dict):
    """name -> Group or numpy array."""

    def require(self, path: str) -> "Group":
        g = self
        for part in [p for p in path.split("/") if p]:
            if part not in g:
                g[part] = Group()
            g = g[part]
            if not isinstance(g, Group):
                raise H5Error(f"{path}: {part} is a dataset")
        return g

    def get_path(self, path: str):
        g = self
        for part in [p for p in path.split("/") if p]:
            if not isinstance(g, Group) or part not in g:
                return None
            g = g[part]
        return g


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ---------------------------------------------------------------- writer --
def _datatype_msg(dt: np.dtype) -> bytes:
    dt = np.dtype(dt)
    if dt.kind in "iu":
        bits = 0x08 if dt.kind == "i" else 0x00
        head = bytes([0x10 | 0, bits, 0, 0]) + struct.pack("<I", dt.itemsize)
        return head + struct.pack("<HH", 0, dt.itemsize * 8)
    if dt.kind == "f":
        if dt.itemsize == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            sign = 63
        elif dt.itemsize == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            sign = 31
        else:
            raise H5Error(f"unsupported float size {dt.itemsize}")
        return bytes([0x10 | 1, 0x20, sign, 0]) + struct.pack("<I", dt.itemsize) + props
    if dt.kind == "c":
        part = np.dtype(f"<f{dt.itemsize // 2}")
        sub = _datatype_msg(part)
        members = b""
        for k, name in enumerate((b"r", b"i")):
            nm = name + b"\0"
            nm += b"\0" * (_pad8(len(nm)) - len(nm))
            members += nm + struct.pack("<IB3xI4x", k * part.itemsize, 0, 0) + b"\0" * 16 + sub
        return bytes([0x10 | 6, 2, 0, 0]) + struct.pack("<I", dt.itemsize) + members
    raise H5Error(f"unsupported dtype {dt}")


def _message(mtype: int, data: bytes, flags: int = 0) -> bytes:
    padded = data + b"\0" * (_pad8(len(data)) - len(data))
    return struct.pack("<HHB3x", mtype, len(padded), flags) + padded


def _object_header(messages: list[bytes]) -> bytes:
    body = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body


class _Writer:
    def __init__(self):
        self.buf = bytearray(96)  # superblock, filled in last

    def tell(self) -> int:
        return len(self.buf)

    def put(self, data: bytes) -> int:
        addr = self.tell()
        self.buf += data
        self.buf += b"\0" * (_pad8(len(self.buf)) - len(self.buf))
        return addr

    def dataset(self, arr: np.ndarray) -> int:
        arr = np.asarray(arr)
        if arr.ndim == 0:
            arr = arr.reshape(1)
        dt = arr.dtype
        if dt.kind == "b":
            arr = arr.astype(np.uint8)
        elif dt.kind == "c":
            arr = arr.astype(np.complex128 if dt.itemsize == 16 else np.complex64)
        arr = np.ascontiguousarray(arr, dtype=arr.dtype.newbyteorder("<"))
        raw = arr.tobytes()
        data_addr = self.put(raw) if raw else UNDEF
        space = struct.pack("<BBBB4x", 1, arr.ndim, 0, 0) + b"".join(struct.pack("<Q", d) for d in arr.shape)
        msgs = [
            _message(0x0001, space),
            _message(0x0003, _datatype_msg(arr.dtype), flags=1),
            _message(0x0005, bytes([2, 2, 2, 0])),
            _message(0x0008, struct.pack("<BBQQ", 3, 1, data_addr, len(raw))),
        ]
        return self.put(_object_header(msgs))

    def group(self, g: Group) -> tuple[int, int, int]:
        names = sorted(g.keys(), key=lambda s: s.encode())
        if len(names) > 2 * GROUP_LEAF_K * 2 * GROUP_INTERNAL_K:
            raise H5Error("more than 256 members in one group")
        entries = []
        for name in names:
            child = g[name]
            if isinstance(child, Group):
                oh, bt, hp = self.group(child)
                entries.append((name, oh, 1, struct.pack("<QQ", bt, hp)))
            else:
                entries.append((name, self.dataset(child), 0, b"\0" * 16))
        # local heap of link names; offset 0 holds the empty name
        heap = bytearray(8)
        offsets = []
        for name in names:
            offsets.append(len(heap))
            nm = name.encode() + b"\0"
            heap += nm + b"\0" * (_pad8(len(nm)) - len(nm))
        free_at = len(heap)
        heap += struct.pack("<QQ", FREE_NULL, 16)  # one free block closes the segment
        heap_data = self.put(bytes(heap))
        heap_addr = self.put(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), free_at, heap_data))
        # symbol-table nodes of up to 2 * leaf K entries, in name order
        cap = 2 * GROUP_LEAF_K
        snods = []
        for s in range(0, len(entries), cap):  # an empty group has an empty B-tree
            chunk = entries[s:s + cap]
            node = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, len(chunk)))
            for (name, oh, ctype, scratch), off in zip(chunk, offsets[s:s + cap]):
                node += struct.pack("<QQI4x", off, oh, ctype) + scratch
            node += b"\0" * (8 + cap * 40 - len(node))
            last = offsets[s + len(chunk) - 1]
            snods.append((self.put(bytes(node)), last))
        # one leaf B-tree node over the symbol-table nodes
        two_k = 2 * GROUP_INTERNAL_K
        tree = bytearray(b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods), UNDEF, UNDEF))
        tree += struct.pack("<Q", 0)
        for addr, last in snods:
            tree += struct.pack("<QQ", addr, last)
        tree += b"\0" * (24 + (2 * two_k + 1) * 8 - len(tree))
        btree_addr = self.put(bytes(tree))
        oh = self.put(_object_header([_message(0x0011, struct.pack("<QQ", btree_addr, heap_addr))]))
        return oh, btree_addr, heap_addr

    def finish(self, root: Group) -> bytes:
        oh, bt, hp = self.group(root)
        eof = self.tell()
        sb = SIGNATURE + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, GROUP_LEAF_K, GROUP_INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
        sb += struct.pack("<QQI4xQQ", 0, oh, 1, bt, hp)
        assert len(sb) == 96
        self.buf[:96] = sb
        return bytes(self.buf)


def write(path: str, root: Group) -> None:
    """Writes the tree to path (atomically: a temporary file is renamed)."""
    data = _Writer().finish(root)
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(data)
    os.replace(tmp, path)


# ---------------------------------------------------------------- reader --
class _Reader:
    def __init__(self, data: bytes):
        self.d = data

    def u(self, fmt: str, off: int):
        return struct.unpack_from("<" + fmt, self.d, off)

    def superblock(self) -> int:
        if self.d[:8] != SIGNATURE:
            raise H5Error("not an HDF5 file (no superblock at offset 0)")
        ver = self.d[8]
        if ver not in (0, 1):
            raise H5Error(f"superblock version {ver} is not supported")
        so, sl = self.d[13], self.d[14]
        if so != 8 or sl != 8:
            raise H5Error("only 8-byte offsets and lengths are supported")
        off = 24 + (4 if ver == 1 else 0)
        off += 32  # base, free space, eof, driver
        _, oh, _, _, _ = self.u("QQI4xQQ", off)
        return oh

    def messages(self, addr: int) -> list[tuple[int, bytes]]:
        if self.d[addr:addr + 4] == b"OHDR":
            raise H5Error("version-2 object headers are not supported")
        ver, _, nmsg, _, size = self.u("BBHII", addr)
        if ver != 1:
            raise H5Error(f"object header version {ver} is not supported")
        out = []
        chunks = [(addr + 16, size)]
        while chunks and len(out) < nmsg:
            start, length = chunks.pop(0)
            p = start
            while p + 8 <= start + length and len(out) < nmsg:
                mtype, msize, _ = self.u("HHB", p)
                body = self.d[p + 8:p + 8 + msize]
                p += 8 + msize
                if mtype == 0x0010:  # continuation
                    caddr, clen = struct.unpack_from("<QQ", body, 0)
                    chunks.append((caddr, clen))
                out.append((mtype, body))
        return out

    def heap_data(self, addr: int) -> int:
        if self.d[addr:addr + 4] != b"HEAP":
            raise H5Error("bad local heap signature")
        _, _, _, data = self.u("B3xQQQ", addr + 4)
        return data

    def name(self, heap_data: int, off: int) -> str:
        end = self.d.index(b"\0", heap_data + off)
        return self.d[heap_data + off:end].decode()

    def group(self, btree: int, heap: int) -> Group:
        g = Group()
        hd = self.heap_data(heap)
        for snod in self.leaves(btree):
            if self.d[snod:snod + 4] != b"SNOD":
                raise H5Error("bad symbol table node signature")
            (n,) = self.u("H", snod + 6)
            for k in range(n):
                e = snod + 8 + 40 * k
                noff, oh, ctype = self.u("QQI", e)
                g[self.name(hd, noff)] = self.object(oh)
        return g

    def leaves(self, addr: int) -> list[int]:
        if self.d[addr:addr + 4] != b"TREE":
            raise H5Error("bad B-tree signature")
        ntype, level, used = self.u("BBH", addr + 4)
        if ntype != 0:
            raise H5Error("not a group B-tree")
        p = addr + 24
        children = []
        for i in range(used):
            (child,) = self.u("Q", p + 8 + 16 * i)
            children.append(child)
        if level == 0:
            return children
        out = []
        for c in children:
            out += self.leaves(c)
        return out

    def object(self, addr: int):
        msgs = self.messages(addr)
        kinds = {t: b for t, b in msgs}
        if 0x0011 in kinds:
            bt, hp = struct.unpack_from("<QQ", kinds[0x0011], 0)
            return self.group(bt, hp)
        if 0x0001 in kinds and 0x0003 in kinds and 0x0008 in kinds:
            return self.dataset(kinds[0x0001], kinds[0x0003], kinds[0x0008])
        if 0x0002 in kinds or 0x000A in kinds:
            raise H5Error("new-style (link-message) groups are not supported")
        raise H5Error(f"object at {addr} is neither a group nor a dataset")

    @staticmethod
    def dtype(b: bytes) -> np.dtype:
        cls, ver = b[0] & 0x0F, b[0] >> 4
        bits0 = b[1]
        (size,) = struct.unpack_from("<I", b, 4)
        order = ">" if bits0 & 1 else "<"
        if cls == 0:
            return np.dtype(f"{order}{'i' if bits0 & 0x08 else 'u'}{size}")
        if cls == 1:
            return np.dtype(f"{order}f{size}")
        if cls == 6:
            nmemb = b[1] | (b[2] << 8)
            p = 8
            fields = []
            for _ in range(nmemb):
                end = b.index(b"\0", p)
                name = b[p:end].decode()
                if ver < 3:
                    p = p + _pad8(end - p + 1)
                else:
                    p = end + 1
                if ver == 1:
                    (off,) = struct.unpack_from("<I", b, p)
                    p += 32  # offset, rank, reserved, permutation, reserved, 4 sizes
                elif ver == 2:
                    (off,) = struct.unpack_from("<I", b, p)
                    p += 4
                else:
                    nb = max(1, (size.bit_length() + 7) // 8)
                    off = int.from_bytes(b[p:p + nb], "little")
                    p += nb
                sub = _Reader.dtype(b[p:])
                p += _Reader.dtype_len(b[p:])
                fields.append((name, off, sub))
            names = [f[0] for f in fields]
            if names == ["r", "i"] and fields[0][2] == fields[1][2] and fields[0][2].kind == "f":
                return np.dtype(f"{fields[0][2].byteorder if fields[0][2].byteorder in '<>' else '<'}c{2 * fields[0][2].itemsize}")
            return np.dtype({"names": names, "formats": [f[2] for f in fields], "offsets": [f[1] for f in fields],
                             "itemsize": size})
        raise H5Error(f"datatype class {cls} is not supported")

    @staticmethod
    def dtype_len(b: bytes) -> int:
        cls = b[0] & 0x0F
        if cls == 0:
            return 12
        if cls == 1:
            return 20
        raise H5Error("nested compound members must be numbers")

    def dataset(self, space: bytes, dtb: bytes, layout: bytes) -> np.ndarray:
        sver, rank, flags = space[0], space[1], space[2]
        p = 8 if sver == 1 else 4
        dims = [struct.unpack_from("<Q", space, p + 8 * k)[0] for k in range(rank)]
        dt = self.dtype(dtb)
        lver = layout[0]
        n = int(np.prod(dims)) if dims else 1
        if lver == 3:
            lclass = layout[1]
            if lclass == 1:
                addr, size = struct.unpack_from("<QQ", layout, 2)
                raw = b"" if addr == UNDEF else self.d[addr:addr + size]
            elif lclass == 0:
                (size,) = struct.unpack_from("<H", layout, 2)
                raw = layout[4:4 + size]
            else:
                raise H5Error("chunked datasets are not supported")
        elif lver in (1, 2):
            lrank, lclass = layout[1], layout[2]
            if lclass != 1:
                raise H5Error("only contiguous version-1/2 layouts are supported")
            (addr,) = struct.unpack_from("<Q", layout, 8)
            raw = self.d[addr:addr + n * dt.itemsize]
        else:
            raise H5Error(f"layout version {lver} is not supported")
        if len(raw) < n * dt.itemsize:
            return np.zeros(dims, dtype=dt)  # never written (fill value zero)
        return np.frombuffer(raw, dtype=dt, count=n).reshape(dims).copy()


def read(path: str) -> Group:
    with open(path, "rb") as f:
        data = f.read()
    r = _Reader(data)
    root_oh = r.superblock()
    root = r.object(root_oh)
    if not isinstance(root, Group):
        raise H5Error("root object is not a group")
    return root
