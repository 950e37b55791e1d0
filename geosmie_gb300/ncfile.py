"""NetCDF classic-format files without the netCDF library.

The optics tables (dointegration.createNCDF, the band files of
bandaverage.fun, the hydrophobic conversion) are NetCDF files; netCDF4 and
h5py are not available where this package runs, so this module writes and
reads the classic format itself, from its published specification (the
"NetCDF Classic Format Specification": header = magic, record count,
dimension list, global attributes, variable list with shapes, attributes,
types, sizes and data offsets; big-endian data of each variable after the
header).  Versions: 1 (classic), 2 (64-bit offsets) and 5 (CDF-5: 64-bit
sizes and the NC_INT64 type).  Any netCDF reader opens these files through
the same API as NETCDF4 files.

Version 2 (the default) has no 64-bit integer type; 'i8' variables are
stored as NC_INT there and as NC_INT64 in version 5.  Record (unlimited)
dimensions are not written.
"""
import struct

import numpy as np

NC_DIMENSION, NC_VARIABLE, NC_ATTRIBUTE = 0x0A, 0x0B, 0x0C
NC_BYTE, NC_CHAR, NC_SHORT, NC_INT, NC_FLOAT, NC_DOUBLE = 1, 2, 3, 4, 5, 6
NC_UBYTE, NC_USHORT, NC_UINT, NC_INT64, NC_UINT64 = 7, 8, 9, 10, 11

_NP = {NC_BYTE: ">i1", NC_CHAR: "S1", NC_SHORT: ">i2", NC_INT: ">i4", NC_FLOAT: ">f4", NC_DOUBLE: ">f8",
       NC_UBYTE: ">u1", NC_USHORT: ">u2", NC_UINT: ">u4", NC_INT64: ">i8", NC_UINT64: ">u8"}
_SIZE = {NC_BYTE: 1, NC_CHAR: 1, NC_SHORT: 2, NC_INT: 4, NC_FLOAT: 4, NC_DOUBLE: 8, NC_UBYTE: 1, NC_USHORT: 2,
         NC_UINT: 4, NC_INT64: 8, NC_UINT64: 8}


def _nc_type(code, version):
    """nc_type of a numpy-style type code ('f8', 'f4', 'i4', 'i8', 'c', ...)."""
    t = {"f8": NC_DOUBLE, "f4": NC_FLOAT, "i4": NC_INT, "i2": NC_SHORT, "i1": NC_BYTE, "c": NC_CHAR, "S1": NC_CHAR,
         "u1": NC_UBYTE, "u2": NC_USHORT, "u4": NC_UINT, "i8": NC_INT64, "u8": NC_UINT64}[code]
    if version != 5 and t == NC_INT64:
        t = NC_INT
    if version != 5 and t > NC_DOUBLE:
        raise ValueError("type %s needs version 5 (CDF-5)" % code)
    return t


def _pad4(n):
    return (4 - n % 4) % 4


class _Writer:
    def __init__(self, version):
        self.v = version
        self.buf = bytearray()

    def i32(self, x):
        self.buf += struct.pack(">i", x)

    def nonneg(self, x):
        self.buf += struct.pack(">q" if self.v == 5 else ">i", x)

    def offset(self, x):
        self.buf += struct.pack(">i" if self.v == 1 else ">q", x)

    def name(self, s):
        b = s.encode("utf-8")
        self.nonneg(len(b))
        self.buf += b + b"\0" * _pad4(len(b))

    def values(self, t, data):
        raw = np.ascontiguousarray(np.asarray(data).astype(_NP[t])).tobytes()
        self.buf += raw + b"\0" * _pad4(len(raw))

    def attrs(self, attrs):
        if not attrs:
            self.i32(0)
            self.nonneg(0)
            return
        self.i32(NC_ATTRIBUTE)
        self.nonneg(len(attrs))
        for k, val in attrs.items():
            self.name(k)
            if isinstance(val, str):
                b = val.encode("utf-8")
                self.i32(NC_CHAR)
                self.nonneg(len(b))
                self.buf += b + b"\0" * _pad4(len(b))
            else:
                a = np.atleast_1d(np.asarray(val))
                t = NC_DOUBLE if a.dtype.kind == "f" else NC_INT
                self.i32(t)
                self.nonneg(a.size)
                self.values(t, a)


def write(path, dims, variables, gattrs=None, version=2):
    """Write a NetCDF classic file.

    dims: ordered [(name, size)]; variables: ordered [(name, type code,
    dimension names, data, {attribute: value})]; text data of 'c' variables
    may be given as a list of strings (padded with NUL to the last
    dimension)."""
    if version not in (1, 2, 5):
        raise ValueError("version must be 1, 2 or 5")
    dim_index = {n: i for i, (n, _) in enumerate(dims)}
    dim_size = dict(dims)
    prepared = []
    for name, code, vdims, data, attrs in variables:
        t = _nc_type(code, version)
        shape = tuple(dim_size[d] for d in vdims)
        if t == NC_CHAR:
            if isinstance(data, (list, tuple)) and data and isinstance(data[0], str):
                arr = np.zeros(shape, dtype="S1")
                for i, s in enumerate(data):
                    b = s.encode("utf-8")[:shape[-1]]
                    arr[i, :len(b)] = np.frombuffer(b, dtype="S1")
                data = arr
            arr = np.asarray(data, dtype="S1").reshape(shape)
        else:
            arr = np.asarray(data).reshape(shape)
        nbytes = int(np.prod(shape, dtype=np.int64)) * _SIZE[t]
        prepared.append((name, t, vdims, arr, attrs or {}, nbytes + _pad4(nbytes)))

    def header(begins):
        w = _Writer(version)
        w.buf += b"CDF" + bytes([version])
        w.nonneg(0)   # no record dimension
        if dims:
            w.i32(NC_DIMENSION)
            w.nonneg(len(dims))
            for n, size in dims:
                w.name(n)
                w.nonneg(size)
        else:
            w.i32(0)
            w.nonneg(0)
        w.attrs(gattrs or {})
        if prepared:
            w.i32(NC_VARIABLE)
            w.nonneg(len(prepared))
            for (name, t, vdims, arr, attrs, vsize), begin in zip(prepared, begins):
                w.name(name)
                w.nonneg(len(vdims))
                for d in vdims:
                    w.nonneg(dim_index[d])
                w.attrs(attrs)
                w.i32(t)
                w.nonneg(min(vsize, 2 ** 32 - 1) if version != 5 else vsize)
                w.offset(begin)
        else:
            w.i32(0)
            w.nonneg(0)
        return w.buf

    hlen = len(header([0] * len(prepared)))
    begins = []
    pos = hlen
    for p in prepared:
        begins.append(pos)
        pos += p[5]
    if version == 1 and pos >= 2 ** 31:
        raise ValueError("file too large for version 1; use version 2")
    with open(path, "wb") as fp:
        fp.write(header(begins))
        for name, t, vdims, arr, attrs, vsize in prepared:
            raw = np.ascontiguousarray(arr.astype(_NP[t])).tobytes()
            fp.write(raw)
            fp.write(b"\0" * (vsize - len(raw)))


class _Reader:
    def __init__(self, raw, version):
        self.raw = raw
        self.v = version
        self.p = 4

    def take(self, fmt):
        x = struct.unpack_from(fmt, self.raw, self.p)[0]
        self.p += struct.calcsize(fmt)
        return x

    def i32(self):
        return self.take(">i")

    def nonneg(self):
        return self.take(">q" if self.v == 5 else ">i")

    def offset(self):
        return self.take(">i" if self.v == 1 else ">q")

    def name(self):
        n = self.nonneg()
        s = self.raw[self.p:self.p + n].decode("utf-8")
        self.p += n + _pad4(n)
        return s

    def attrs(self):
        tag = self.i32()
        n = self.nonneg()
        out = {}
        if tag == 0:
            return out
        for _ in range(n):
            k = self.name()
            t = self.i32()
            m = self.nonneg()
            nbytes = m * _SIZE[t]
            chunk = self.raw[self.p:self.p + nbytes]
            self.p += nbytes + _pad4(nbytes)
            if t == NC_CHAR:
                out[k] = chunk.decode("utf-8")
            else:
                a = np.frombuffer(chunk, dtype=_NP[t]).astype(_NP[t][1:])
                out[k] = a if a.size > 1 else a[0]
        return out


def read(path):
    """(dims {name: size}, variables {name: (dims, attrs, data)}, gattrs)."""
    with open(path, "rb") as fp:
        raw = fp.read()
    if raw[:3] != b"CDF" or raw[3] not in (1, 2, 5):
        raise ValueError("not a NetCDF classic file")
    r = _Reader(raw, raw[3])
    r.nonneg()   # record count
    tag = r.i32()
    nd = r.nonneg()
    dims = []
    if tag == NC_DIMENSION:
        for _ in range(nd):
            n = r.name()
            dims.append((n, r.nonneg()))
    gattrs = r.attrs()
    tag = r.i32()
    nv = r.nonneg()
    variables = {}
    if tag == NC_VARIABLE:
        for _ in range(nv):
            name = r.name()
            rank = r.nonneg()
            ids = [r.nonneg() for _ in range(rank)]
            attrs = r.attrs()
            t = r.i32()
            r.nonneg()   # vsize
            begin = r.offset()
            vdims = tuple(dims[i][0] for i in ids)
            shape = tuple(dims[i][1] for i in ids)
            n = int(np.prod(shape, dtype=np.int64))
            data = np.frombuffer(raw, dtype=_NP[t], count=n, offset=begin).reshape(shape)
            data = data if t == NC_CHAR else data.astype(_NP[t][1:])
            variables[name] = (vdims, attrs, data)
    return dict(dims), variables, gattrs
