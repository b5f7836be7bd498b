"""A second, independent reader of the HDF5 subset the checkpoint writer emits,
written from the HDF5 File Format Specification 3.0 for the tests: superblock
version 2/3, version 2 object headers, compact-link groups, contiguous or
compact datasets of little-endian integers, IEEE doubles and variable-length
strings (global heap).  Every checksum (Jenkins lookup3) is verified, and
every structural field the writer sets is checked against the spec's
allowed values, so a file that parses here is well-formed for those parts of
the format."""
from __future__ import annotations

import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


def lookup3(data: bytes, initval: int = 0) -> int:
    """Bob Jenkins' hashlittle, as published in lookup3.c."""
    M = 0xFFFFFFFF

    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & M

    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & M
    i = 0
    while n - i > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & M
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & M
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & M
        a = (a - c) & M; a ^= rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 4); b = (b + a) & M
        i += 12
    rest = data[i:]
    if not rest:
        return c
    rest = rest + bytes(12 - len(rest))
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


class FormatError(ValueError):
    pass


def _req(cond, what):
    if not cond:
        raise FormatError(what)


class File:
    def __init__(self, path: str):
        with open(path, "rb") as f:
            self.b = f.read()
        b = self.b
        _req(b[:8] == b"\x89HDF\r\n\x1a\n", "signature")
        _req(b[8] in (2, 3), "superblock version")
        _req(b[9] == 8 and b[10] == 8, "offset/length sizes")
        _req(lookup3(b[:44]) == struct.unpack_from("<I", b, 44)[0], "superblock checksum")
        base, ext, eof, root = struct.unpack_from("<QQQQ", b, 12)
        _req(base == 0, "base address")
        _req(eof == len(b), "end-of-file address equals the file size")
        self.ext = ext
        self.root = root
        self.headers = {}   # address -> list of (type, flags, data)

    def header(self, addr: int):
        if addr in self.headers:
            return self.headers[addr]
        b = self.b
        _req(b[addr:addr + 4] == b"OHDR" and b[addr + 4] == 2, f"object header at {addr}")
        flags = b[addr + 5]
        _req(flags & 0xC0 == 0, "reserved object header flags")
        at = addr + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
        csz = 1 << (flags & 3)
        chunk = int.from_bytes(b[at:at + csz], "little")
        at += csz
        end = at + chunk
        _req(lookup3(b[addr:end]) == struct.unpack_from("<I", b, end)[0], f"object header checksum at {addr}")
        msgs = []
        hsz = 6 if flags & 0x04 else 4
        while end - at >= hsz:
            t, sz, mf = b[at], struct.unpack_from("<H", b, at + 1)[0], b[at + 3]
            _req(at + hsz + sz <= end, "message overruns its chunk")
            _req(t != 0x10, "continuation messages are not in this subset")
            msgs.append((t, mf, b[at + hsz:at + hsz + sz]))
            at += hsz + sz
        self.headers[addr] = msgs
        return msgs

    def links(self, addr: int) -> dict:
        msgs = self.header(addr)
        types = [t for t, _, _ in msgs]
        _req(0x02 in types and 0x0A in types, "a group holds link info and group info messages")
        for t, _, d in msgs:
            if t == 0x02:
                _req(d[0] == 0, "link info version")
                at = 2 + (8 if d[1] & 1 else 0)
                heap, bt = struct.unpack_from("<QQ", d, at)
                _req(heap == UNDEF and bt == UNDEF, "compact storage: no fractal heap, no name index")
            if t == 0x0A:
                _req(d[0] == 0, "group info version")
                if d[1] & 1:
                    maxc, mind = struct.unpack_from("<HH", d, 2)
                    _req(mind <= maxc + 1, "phase change values")
        out = {}
        for t, _, d in msgs:
            if t != 0x06:
                continue
            _req(d[0] == 1, "link message version")
            fl = d[1]
            at = 2
            ltype = 0
            if fl & 0x08:
                ltype = d[at]; at += 1
            if fl & 0x04:
                at += 8
            if fl & 0x10:
                at += 1
            lsz = 1 << (fl & 3)
            n = int.from_bytes(d[at:at + lsz], "little"); at += lsz
            name = d[at:at + n].decode("ascii"); at += n
            _req(ltype == 0, "hard links only")
            _req(name not in out, "duplicate link name")
            out[name] = struct.unpack_from("<Q", d, at)[0]
        return out

    def resolve(self, path: str) -> int:
        addr = self.root
        for part in [p for p in path.split("/") if p]:
            links = self.links(addr)
            if part not in links:
                raise KeyError(path)
            addr = links[part]
        return addr

    def is_group(self, path: str) -> bool:
        return any(t == 0x02 for t, _, _ in self.header(self.resolve(path)))

    def keys(self, path: str = "/") -> list:
        return sorted(self.links(self.resolve(path)))

    def dataset(self, path: str):
        msgs = self.header(self.resolve(path))
        shape = dtype = layout = None
        for t, _, d in msgs:
            if t == 0x01:
                ver, rank, fl = d[0], d[1], d[2]
                _req(ver in (1, 2), "dataspace version")
                at = 8 if ver == 1 else 4
                if ver == 2:
                    _req(d[3] in (0, 1), "scalar or simple dataspace")
                shape = struct.unpack_from("<" + "Q" * rank, d, at)
                if fl & 1:
                    mx = struct.unpack_from("<" + "Q" * rank, d, at + 8 * rank)
                    _req(all(m >= s for m, s in zip(mx, shape)), "max dims")
            elif t == 0x03:
                cls, ver = d[0] & 0x0F, d[0] >> 4
                size = struct.unpack_from("<I", d, 4)[0]
                _req(ver == 1, "datatype version 1")
                if cls == 0:
                    _req(d[1] & 1 == 0, "little-endian integers")
                    off, prec = struct.unpack_from("<HH", d, 8)
                    _req(off == 0 and prec == 8 * size, "integer precision")
                    dtype = np.dtype(("<i" if d[1] & 0x08 else "<u") + str(size))
                elif cls == 1:
                    _req(d[1] == 0x20 and d[2] == 63 and size == 8, "IEEE double bit field")
                    off, prec, eloc, esz, mloc, msz, bias = struct.unpack_from("<HHBBBBI", d, 8)
                    _req((off, prec, eloc, esz, mloc, msz, bias) == (0, 64, 52, 11, 0, 52, 1023),
                         "IEEE double properties")
                    dtype = np.dtype("<f8")
                elif cls == 9:
                    _req(d[1] & 0x0F == 1 and size == 16, "variable-length string")
                    base = d[8:]
                    _req(base[0] == 0x10 and struct.unpack_from("<I", base, 4)[0] == 1, "string base type")
                    dtype = "vstr"
                else:
                    raise FormatError(f"datatype class {cls}")
            elif t == 0x05:
                _req(d[0] in (1, 2, 3), "fill value version")
                if d[0] == 2:
                    _req(d[1] in (1, 2, 3) and d[2] in (0, 1, 2) and d[3] in (0, 1), "fill value fields")
                    _req(len(d) == (4 if d[3] == 0 else 8 + struct.unpack_from("<I", d, 4)[0]),
                         "fill value size")
            elif t == 0x08:
                _req(d[0] == 3, "layout version 3")
                if d[1] == 1:
                    layout = ("contiguous",) + struct.unpack_from("<QQ", d, 2)
                elif d[1] == 0:
                    n = struct.unpack_from("<H", d, 2)[0]
                    layout = ("compact", d[4:4 + n])
                else:
                    raise FormatError("chunked layout")
        _req(shape is not None and dtype is not None and layout is not None, "dataset messages")
        n = int(np.prod(shape)) if shape else 1
        esz = 16 if dtype == "vstr" else dtype.itemsize
        if layout[0] == "contiguous":
            addr, size = layout[1], layout[2]
            _req(size == n * esz, "contiguous size = elements x element size")
            raw = bytes(size) if addr == UNDEF else self.b[addr:addr + size]
            _req(addr == UNDEF or addr + size <= len(self.b), "data inside the file")
        else:
            raw = layout[1]
        if dtype == "vstr":
            return np.array([self._vstr(raw[16 * i:16 * i + 16]) for i in range(n)],
                            dtype=object).reshape(shape)
        return np.frombuffer(raw, dtype=dtype, count=n).reshape(shape)

    def _vstr(self, el: bytes) -> str:
        length, gaddr, idx = struct.unpack("<IQI", el)
        b = self.b
        _req(b[gaddr:gaddr + 4] == b"GCOL" and b[gaddr + 4] == 1, "global heap collection")
        csize = struct.unpack_from("<Q", b, gaddr + 8)[0]
        _req(csize >= 4096, "global heap collection of at least 4 KiB")
        at = 16
        while at + 16 <= csize:
            oi, _, osz = struct.unpack_from("<HHxxxxQ", b, gaddr + at)
            if oi == 0:
                _req(osz == csize - at, "free space object covers the rest of the collection")
                break
            if oi == idx:
                _req(osz == length, "heap object size = string length")
                return b[gaddr + at + 16:gaddr + at + 16 + length].decode("ascii")
            at += 16 + ((osz + 7) & ~7)
        raise FormatError(f"global heap object {idx} missing")
