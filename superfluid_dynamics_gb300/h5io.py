"""State and trajectory files in the reference's HDF5 layouts, without an HDF5
library (none is installed beside this package).

Layouts:
- State file (SimulationRunner.cuh:99-178, loadStateFile / saveStateFile):
  datasets ``interface`` (N x 2 doubles, the (x, y) pairs of Z) and
  ``potential`` (N doubles), root attributes ``rho``, ``kappa``, ``U``,
  ``depth``, ``initial_amplitude`` (doubles) and ``rhs`` (bool).
- Simulation file (Python/simulation.py:97-130, saveSimulationFile /
  loadSimulationFile): datasets ``T``, ``Y``, ``Y0``, root attributes
  ``depth``, ``L``, ``N``, ``t0``, ``t1``, ``initial_amplitude``, ``g``.

The files are written in the subset of the HDF5 format that libhdf5 itself
writes with its default (earliest) format settings (h5py and HighFive read
that subset; neither is installed beside this package, so the check is
byte-level against libhdf5-written files):
- version-0 superblock with 8-byte offsets and lengths;
- version-1 object headers;
- the root group as a symbol table (local heap, one version-1 B-tree leaf,
  one symbol-table node);
- contiguous datasets of little-endian IEEE doubles or 64-bit integers;
- version-1 attribute messages with scalar dataspaces.
Booleans are the enum {FALSE = 0, TRUE = 1} over a signed byte, as h5py and
HighFive store them.  The reader covers that subset, plus continuation and NIL
messages, for files from other writers that keep to it.
"""
from __future__ import annotations

import math
import os
import struct

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF
_HEAP_FREE_NULL = 1          # end of a local heap's free list
_LEAF_K, _INTERNAL_K = 4, 16  # group B-tree parameters of the superblock

# message types
_NIL, _DATASPACE, _DATATYPE, _FILL, _LAYOUT, _ATTR, _CONT, _SYMTAB = 0x0, 0x1, 0x3, 0x5, 0x8, 0xC, 0x10, 0x11


class H5FormatError(ValueError):
    """The file is not HDF5, or uses a part of the format outside this subset."""


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ------------------------------------------------------------------ encoding
def _dtype_msg(dt: np.dtype) -> bytes:
    dt = np.dtype(dt)
    if dt == np.float64:
        # class 1 (floating point), version 1; little endian, implied mantissa
        # normalisation, sign at bit 63; offset 0, precision 64, exponent at
        # 52 (11 bits), mantissa at 0 (52 bits), bias 1023
        return bytes([0x11, 0x20, 0x3F, 0x00]) + struct.pack("<IHHBBBBI", 8, 0, 64, 52, 11, 0, 52, 1023)
    if dt == np.int64:
        # class 0 (fixed point), version 1, little endian, signed
        return bytes([0x10, 0x08, 0x00, 0x00]) + struct.pack("<IHH", 8, 0, 64)
    if dt == np.bool_:
        # class 8 (enum), version 1, 2 members over a signed byte
        base = bytes([0x10, 0x08, 0x00, 0x00]) + struct.pack("<IHH", 1, 0, 8)
        names = b"FALSE".ljust(8, b"\0") + b"TRUE".ljust(8, b"\0")
        return bytes([0x18, 0x02, 0x00, 0x00]) + struct.pack("<I", 1) + base + names + bytes([0, 1])
    raise H5FormatError(f"unsupported element type {dt}")


def _dataspace_msg(shape: tuple, maxdims: bool) -> bytes:
    rank = len(shape)
    out = struct.pack("<BBBBI", 1, rank, 1 if (maxdims and rank) else 0, 0, 0)
    out += b"".join(struct.pack("<Q", d) for d in shape)
    if maxdims and rank:
        out += b"".join(struct.pack("<Q", d) for d in shape)
    return out


def _message(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = body.ljust(_pad8(len(body)), b"\0")
    return struct.pack("<HHBxxx", mtype, len(body), flags) + body


def _object_header(messages: list) -> bytes:
    data = b"".join(messages)
    return struct.pack("<BBHII", 1, 0, len(messages), 1, len(data)) + b"\0" * 4 + data


def _attr_msg(name: str, value) -> bytes:
    if isinstance(value, (bool, np.bool_)):
        dt, raw = np.dtype(np.bool_), struct.pack("<b", 1 if value else 0)
    elif isinstance(value, (int, np.integer)):
        dt, raw = np.dtype(np.int64), struct.pack("<q", int(value))
    else:
        dt, raw = np.dtype(np.float64), struct.pack("<d", float(value))
    nm = name.encode() + b"\0"
    dtm, dsm = _dtype_msg(dt), _dataspace_msg((), False)
    body = struct.pack("<BBHHH", 1, 0, len(nm), len(dtm), len(dsm))
    body += nm.ljust(_pad8(len(nm)), b"\0") + dtm.ljust(_pad8(len(dtm)), b"\0") + dsm.ljust(_pad8(len(dsm)), b"\0")
    return _message(_ATTR, body + raw)


def write(path: str, datasets: dict, attrs: dict | None = None) -> None:
    """Write `datasets` (name -> array of float64 or int64) and root `attrs`
    (name -> float, int or bool) as an HDF5 file."""
    attrs = attrs or {}
    if not datasets:
        raise H5FormatError("at least one dataset is required")
    if len(datasets) > 2 * _LEAF_K:
        raise H5FormatError(f"at most {2 * _LEAF_K} datasets per file")
    arrs = {}
    for k, v in datasets.items():
        a = np.ascontiguousarray(v)
        if a.dtype.kind == "f":
            a = a.astype("<f8")
        elif a.dtype.kind in "iu":
            a = a.astype("<i8")
        else:
            raise H5FormatError(f"dataset {k}: unsupported element type {a.dtype}")
        arrs[k] = a
    names = list(arrs)
    # local heap data: the empty name at 0, then each name, 8-byte aligned
    heap = b"\0" * 8
    offs = {}
    for k in names:
        offs[k] = len(heap)
        heap += (k.encode() + b"\0").ljust(_pad8(len(k) + 1), b"\0")
    root_msgs_len = len(_message(_SYMTAB, b"\0" * 16)) + sum(len(_attr_msg(k, v)) for k, v in attrs.items())
    # layout: superblock | root header | B-tree | heap header | heap data | SNOD | dataset headers | data
    a_root = 96
    a_btree = a_root + 16 + root_msgs_len
    btree_size = 24 + (2 * _INTERNAL_K + 1) * 8 + 2 * _INTERNAL_K * 8
    a_heap = a_btree + btree_size
    a_heapdata = a_heap + 32
    a_snod = a_heapdata + len(heap)
    snod_size = 8 + 2 * _LEAF_K * 40

    def dataset_header(a: np.ndarray, addr: int) -> bytes:
        return _object_header([
            _message(_DATASPACE, _dataspace_msg(a.shape, True)),
            _message(_DATATYPE, _dtype_msg(a.dtype), flags=1),
            _message(_FILL, bytes([2, 2, 2, 1, 0, 0, 0, 0]), flags=1),  # version 2: late, if set, default value
            _message(_LAYOUT, struct.pack("<BBQQ", 3, 1, addr, a.nbytes))])  # version 3, contiguous

    pos = a_snod + snod_size
    hdr_addr, data_addr = {}, {}
    for k in names:  # header sizes do not depend on the data address
        hdr_addr[k] = pos
        pos = _pad8(pos + len(dataset_header(arrs[k], 0)))
    for k in names:
        data_addr[k] = pos
        pos = _pad8(pos + arrs[k].nbytes)
    eof = pos
    hdrs = {k: dataset_header(arrs[k], data_addr[k]) for k in names}
    root = _object_header([_message(_SYMTAB, struct.pack("<QQ", a_btree, a_heap))] +
                          [_attr_msg(k, v) for k, v in attrs.items()])
    assert len(root) == 16 + root_msgs_len
    sorted_names = sorted(names, key=lambda s: s.encode())
    btree = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, _UNDEF, _UNDEF)
    btree += struct.pack("<QQQ", 0, a_snod, offs[sorted_names[-1]])
    btree = btree.ljust(btree_size, b"\0")
    heap_hdr = b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap), _HEAP_FREE_NULL, a_heapdata)
    snod = b"SNOD" + struct.pack("<BBH", 1, 0, len(names))
    for k in sorted_names:
        snod += struct.pack("<QQII", offs[k], hdr_addr[k], 0, 0) + b"\0" * 16
    snod = snod.ljust(snod_size, b"\0")
    sb = _SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", _LEAF_K, _INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
    sb += struct.pack("<QQII", 0, a_root, 1, 0) + struct.pack("<QQ", a_btree, a_heap)
    assert len(sb) == 96
    buf = bytearray(eof)
    for addr, blob in [(0, sb), (a_root, root), (a_btree, btree), (a_heap, heap_hdr), (a_heapdata, heap),
                       (a_snod, snod)] + [(hdr_addr[k], hdrs[k]) for k in names] + \
                      [(data_addr[k], arrs[k].tobytes()) for k in names]:
        buf[addr:addr + len(blob)] = blob
    with open(path, "wb") as f:
        f.write(bytes(buf))


# ------------------------------------------------------------------ decoding
class _Reader:
    def __init__(self, b: bytes):
        self.b = b

    def u(self, fmt: str, off: int):
        return struct.unpack_from("<" + fmt, self.b, off)

    def messages(self, addr: int):
        ver, _, nmsg, _, size = self.u("BBHII", addr)
        if ver != 1:
            raise H5FormatError(f"object header version {ver} at {addr}")
        out, chunks = [], [(addr + 16, size)]
        while chunks and len(out) < nmsg:
            p, n = chunks.pop(0)
            end = p + n
            while p + 8 <= end and len(out) < nmsg:
                t, sz, fl = self.u("HHB", p)
                body = self.b[p + 8:p + 8 + sz]
                if t == _CONT:
                    chunks.append(struct.unpack_from("<QQ", body))
                out.append((t, body, fl))
                p += 8 + sz
        return out

    @staticmethod
    def dataspace(body: bytes):
        ver, rank, flags = body[0], body[1], body[2]
        p = 8 if ver == 1 else 4
        if ver not in (1, 2):
            raise H5FormatError(f"dataspace version {ver}")
        return tuple(struct.unpack_from("<Q", body, p + 8 * i)[0] for i in range(rank))

    @staticmethod
    def dtype(body: bytes):
        cls, ver = body[0] & 0x0F, body[0] >> 4
        bits = body[1] | (body[2] << 8) | (body[3] << 16)
        size = struct.unpack_from("<I", body, 4)[0]
        order = ">" if bits & 1 else "<"
        if cls == 1 and size in (4, 8):
            return np.dtype(order + ("f4" if size == 4 else "f8"))
        if cls == 0 and size in (1, 2, 4, 8):
            return np.dtype(order + ("i" if bits & 0x08 else "u") + str(size))
        if cls == 8:
            base = _Reader.dtype(body[8:])
            nmem = bits & 0xFFFF
            p = 8 + 12
            names = []
            for _ in range(nmem):
                e = body.index(b"\0", p)
                names.append(body[p:e].decode())
                p += _pad8(e - p + 1) if ver < 3 else e - p + 1
            if sorted(names) == ["FALSE", "TRUE"] and base.itemsize == 1:
                return np.dtype(np.bool_)
            return base
        raise H5FormatError(f"datatype class {cls} size {size}")

    def attribute(self, body: bytes):
        ver = body[0]
        if ver != 1:
            raise H5FormatError(f"attribute message version {ver}")
        nlen, dlen, slen = struct.unpack_from("<HHH", body, 2)
        p = 8
        name = body[p:p + nlen - 1].decode()
        p += _pad8(nlen)
        dt = self.dtype(body[p:p + dlen])
        p += _pad8(dlen)
        shape = self.dataspace(body[p:p + slen])
        p += _pad8(slen)
        count = int(np.prod(shape)) if shape else 1
        raw = np.frombuffer(body, dtype=np.int8 if dt == np.bool_ else dt, count=count, offset=p)
        val = raw.astype(bool) if dt == np.bool_ else raw
        val = val.reshape(shape) if shape else val[0]
        return name, (val.item() if not shape else val.copy())


def read(path: str):
    """Datasets (name -> array) and root attributes (name -> value) of an HDF5
    file in the subset this module writes.  A truncated or malformed file
    raises H5FormatError."""
    with open(path, "rb") as f:
        b = f.read()
    try:
        return _read(path, b)
    except H5FormatError:
        raise
    except (struct.error, IndexError, ValueError) as e:  # a field or block outside the file
        raise H5FormatError(f"{path}: truncated or malformed ({e})") from e


def _read(path: str, b: bytes):
    if b[:8] != _SIG:
        raise H5FormatError(f"{path}: not an HDF5 file")
    if b[8] != 0 or b[13] != 8 or b[14] != 8:
        raise H5FormatError(f"{path}: superblock version {b[8]} / offset sizes {b[13]}, {b[14]} not supported")
    R = _Reader(b)
    a_root = R.u("Q", 64)[0]
    attrs, datasets = {}, {}
    btree = heap = None
    for t, body, _ in R.messages(a_root):
        if t == _SYMTAB:
            btree, heap = struct.unpack_from("<QQ", body)
        elif t == _ATTR:
            k, v = R.attribute(body)
            attrs[k] = v
    if btree is None:
        raise H5FormatError(f"{path}: root group is not a symbol-table group")
    if b[heap:heap + 4] != b"HEAP":
        raise H5FormatError(f"{path}: bad local heap")
    hsize, _, hdata = R.u("QQQ", heap + 8)

    def leaves(addr):
        if b[addr:addr + 4] != b"TREE":
            raise H5FormatError(f"{path}: bad B-tree node")
        ntype, level, used = R.u("BBH", addr + 4)
        kids = [R.u("Q", addr + 24 + 8 + 16 * i)[0] for i in range(used)]
        if level == 0:
            return kids
        return [x for k in kids for x in leaves(k)]

    for snod in leaves(btree):
        if b[snod:snod + 4] != b"SNOD":
            raise H5FormatError(f"{path}: bad symbol-table node")
        nsym = R.u("H", snod + 6)[0]
        for i in range(nsym):
            off, oh = R.u("QQ", snod + 8 + 40 * i)
            name = b[hdata + off:b.index(b"\0", hdata + off)].decode()
            shape, dt, addr, size = None, None, None, None
            for t, body, _ in R.messages(oh):
                if t == _DATASPACE:
                    shape = R.dataspace(body)
                elif t == _DATATYPE:
                    dt = R.dtype(body)
                elif t == _LAYOUT:
                    if body[0] != 3 or body[1] != 1:
                        raise H5FormatError(f"{path}: dataset {name}: layout version {body[0]} class {body[1]}")
                    addr, size = struct.unpack_from("<QQ", body, 2)
            if shape is None or dt is None or addr is None:
                continue  # not a dataset (a subgroup): outside this subset
            count = math.prod(shape) if shape else 1  # Python integers: no wrap-around
            if addr == _UNDEF:
                arr = np.zeros(count, dtype=dt)
            else:
                if addr > len(b) or count * dt.itemsize > len(b) - addr:
                    raise H5FormatError(f"{path}: dataset {name} runs past the end of the file")
                arr = np.frombuffer(b, dtype=dt, count=count, offset=addr).copy()
            datasets[name] = arr.reshape(shape).astype(dt.newbyteorder("="))
    return datasets, attrs


# ------------------------------------------------------------------ reference layouts
def save_state_file(path: str, Z, phi, properties: dict, rhs: bool = False) -> int:
    """saveStateFile (SimulationRunner.cuh:144-178): `interface` = (Re Z, Im Z)
    per node, `potential` = phi, root attributes rho, kappa, U, depth,
    initial_amplitude (from `properties`, 0 when absent) and rhs.  Returns 0."""
    Z = np.asarray(Z, dtype=np.complex128)
    phi = np.asarray(phi, dtype=np.float64)
    attrs = {k: float(properties.get(k, 0.0)) for k in ("rho", "kappa", "U", "depth", "initial_amplitude")}
    attrs["rhs"] = bool(rhs)
    write(path, {"interface": np.stack([Z.real, Z.imag], axis=1), "potential": phi}, attrs)
    return 0


def load_state_file(path: str, N: int, scale_y: float = 1.0):
    """loadStateFile (SimulationRunner.cuh:99-142): (Z, phi), Z = x + i scale_y y,
    with the reference's shape checks and messages."""
    ds, _ = read(path)
    if "interface" not in ds or "potential" not in ds:
        raise RuntimeError("the file must hold the datasets 'interface' and 'potential'")
    itf, pot = ds["interface"], ds["potential"]
    if itf.ndim != 2 or itf.shape[1] != 2 or itf.shape[0] != N:
        if itf.ndim == 1:
            raise RuntimeError(f"Interface must have shape ({N}, 2), instead it has ({itf.shape[0]},)")
        if itf.ndim == 2:
            raise RuntimeError(f"Interface must have shape ({N}, 2), instead it has ({itf.shape[0]}, {itf.shape[1]})")
        raise RuntimeError(f"Interface must have shape ({N}, 2), instead it has a higher dimensionality "
                           f"than 2 ({itf.ndim})!")
    if pot.ndim == 0:
        raise RuntimeError("potential dataset is empty.")
    return itf[:, 0] + 1j * scale_y * itf[:, 1], np.asarray(pot, dtype=np.float64).reshape(-1)


def save_simulation_file(filename: str, T, Y, Y0, L: float, depth: float, t0: float, t1: float,
                         initial_amplitude: float, g: float, N: int | None = None) -> None:
    """saveSimulationFile (Python/simulation.py:97-110).  The reference stores a
    module-level N; here it is the argument, or len(Y0) / 3."""
    Y0 = np.asarray(Y0, dtype=np.float64)
    n = int(N) if N is not None else Y0.size // 3
    write(filename, {"T": np.asarray(T, dtype=np.float64), "Y": np.asarray(Y, dtype=np.float64), "Y0": Y0},
          {"depth": float(depth), "L": float(L), "N": n, "t0": float(t0), "t1": float(t1),
           "initial_amplitude": float(initial_amplitude), "g": float(g)})


def load_simulation_file(filename: str):
    """loadSimulationFile (Python/simulation.py:111-130): (T, Y, Y0, L, depth, N,
    t0, t1, initial_amplitude, g), or None when the file does not exist."""
    if not os.path.exists(filename):
        return None
    ds, at = read(filename)
    return (ds["T"], ds["Y"], ds["Y0"], at["L"], at["depth"], at["N"], at["t0"], at["t1"],
            at["initial_amplitude"], at["g"])
