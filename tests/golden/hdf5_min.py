"""Minimal HDF5 reader for the reference's entropy-contribution files --
TEST INFRASTRUCTURE (golden-fixture extraction only).

The reference writes entcontri_*.nc through libnetcdf as NetCDF-4, i.e.
HDF5 (src/Netcdf_EntContri.cpp:577-769, NC_NETCDF4).  No HDF5 library is in
this image, so this restates just enough of the published HDF5 file format
to read those files: version-2 object headers ("OHDR", with "OCHK"
continuation blocks), the dataspace, datatype and data-layout messages, and
chunked storage indexed by a version-1 B-tree ("TREE", node type 1) without
filters.  Datasets are found by scanning the file for object headers and
recognised by rank and element type, because the link names live in a
fractal heap this reader does not parse:

    id        [records][order]                 4-byte unsigned integers
    contri_S  [records][estimators][schemes][steps]   8-byte floats
"""
from __future__ import annotations

import numpy as np

MSG_DATASPACE, MSG_DATATYPE, MSG_LAYOUT, MSG_CONT = 0x0001, 0x0003, 0x0008, 0x0010


class H5Error(ValueError):
    pass


def _u(buf, off, n):
    return int.from_bytes(buf[off:off + n], "little")


def _messages(buf, off):
    """(type, payload) of every message of the object header at off."""
    if buf[off:off + 4] != b"OHDR":
        raise H5Error("not an object header")
    ver, flags = buf[off + 4], buf[off + 5]
    if ver != 2:
        raise H5Error("object header version")
    p = off + 6
    if flags & 0x20:
        p += 16
    if flags & 0x10:
        p += 4
    size_len = 1 << (flags & 3)
    chunk_len = _u(buf, p, size_len)
    p += size_len
    blocks = [(p, p + chunk_len)]
    out = []
    while blocks:
        start, end = blocks.pop(0)
        q = start
        while q + 4 <= end - 4:      # leave room for the checksum
            mtype = buf[q]
            msize = _u(buf, q + 1, 2)
            q += 4 + (2 if flags & 0x04 else 0)
            payload = buf[q:q + msize]
            q += msize
            if mtype == MSG_CONT:
                addr, length = _u(payload, 0, 8), _u(payload, 8, 8)
                if buf[addr:addr + 4] != b"OCHK":
                    raise H5Error("continuation block")
                blocks.append((addr + 4, addr + length))
            elif mtype != 0:
                out.append((mtype, payload))
    return out


def _dataspace(m):
    ver, rank, flags = m[0], m[1], m[2]
    p = 4 if ver == 2 else 8
    return [_u(m, p + 8 * k, 8) for k in range(rank)]


def _datatype(m):
    cls = m[0] & 0x0F
    bits = m[1]
    size = _u(m, 4, 4)
    if cls not in (0, 1):
        return None                      # strings, references ...: not needed here
    order = ">" if bits & 1 else "<"
    if cls == 0:
        signed = bool(bits & 0x08)
        return np.dtype(order + ("i" if signed else "u") + str(size))
    return np.dtype(order + "f" + str(size))


def _layout(m):
    ver = m[0]
    if ver != 3:
        raise H5Error(f"layout message version {ver}")
    cls = m[1]
    if cls == 2:                         # chunked
        nd = m[2]
        addr = _u(m, 3, 8)
        dims = [_u(m, 11 + 4 * k, 4) for k in range(nd)]
        return ("chunked", addr, dims)
    if cls == 1:                         # contiguous
        return ("contiguous", _u(m, 2, 8), _u(m, 10, 8))
    raise H5Error(f"layout class {cls}")


def _chunks(buf, addr, rank):
    """(offsets, chunk address, size) of every chunk under a v1 B-tree."""
    if addr == 0xFFFFFFFFFFFFFFFF:
        return []
    if buf[addr:addr + 4] != b"TREE" or buf[addr + 4] != 1:
        raise H5Error("chunk B-tree")
    level = buf[addr + 5]
    used = _u(buf, addr + 6, 2)
    p = addr + 8 + 16
    key_len = 8 + 8 * (rank + 1)
    out = []
    for _ in range(used):
        size = _u(buf, p, 4)
        offs = [_u(buf, p + 8 + 8 * k, 8) for k in range(rank)]
        child = _u(buf, p + key_len, 8)
        if level == 0:
            out.append((offs, child, size))
        else:
            out.extend(_chunks(buf, child, rank))
        p += key_len + 8
    return out


def datasets(path):
    """Every dataset found in the file: list of numpy arrays."""
    buf = open(path, "rb").read()
    if buf[:8] != b"\x89HDF\r\n\x1a\n":
        raise H5Error("not an HDF5 file")
    found = []
    pos = buf.find(b"OHDR")
    while pos >= 0:
        try:
            msgs = dict((t, m) for t, m in _messages(buf, pos))
        except (H5Error, IndexError):
            msgs = {}
        if MSG_DATASPACE in msgs and MSG_DATATYPE in msgs and MSG_LAYOUT in msgs:
            shape = _dataspace(msgs[MSG_DATASPACE])
            dt = _datatype(msgs[MSG_DATATYPE])
            if dt is None:
                pos = buf.find(b"OHDR", pos + 4)
                continue
            lay = _layout(msgs[MSG_LAYOUT])
            arr = np.zeros(shape, dt)
            if lay[0] == "chunked" and all(s > 0 for s in shape):
                cdims = lay[2][:-1]
                for offs, caddr, size in _chunks(buf, lay[1], len(shape)):
                    n = int(np.prod(cdims)) * dt.itemsize
                    if size != n:
                        raise H5Error("filtered chunk")
                    block = np.frombuffer(buf, dt, int(np.prod(cdims)), caddr).reshape(cdims)
                    sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
                    sub = tuple(slice(0, x.stop - x.start) for x in sl)
                    arr[sl] = block[sub]
            elif (lay[0] == "contiguous" and all(s > 0 for s in shape)
                  and lay[1] != 0xFFFFFFFFFFFFFFFF):
                arr = np.frombuffer(buf, dt, int(np.prod(shape)), lay[1]).reshape(shape).copy()
            found.append(arr)
        pos = buf.find(b"OHDR", pos + 4)
    return found


def read_entcontri(path):
    """(ids [records][order] uint32, contri_S [records][est][sch][steps] f64)."""
    ids = contri = None
    for a in datasets(path):
        if a.ndim == 2 and a.dtype == np.uint32:
            ids = a
        elif a.ndim == 4 and a.dtype == np.float64:
            contri = a
    if ids is None or contri is None:
        raise H5Error(f"{path}: id / contri_S not found")
    return ids, contri
