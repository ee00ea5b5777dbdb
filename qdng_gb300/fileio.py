"""QDng data files: raw binary + `.meta` and the protobuf stream format.

* Raw form (`FileSingle` raw, src/tools/FileSingle.h:1243-1390): the array
  as little-endian bytes in `<name><suffix>` (complex128 for wave functions,
  float64 for grid operators and laser fields) and a key-value text file
  `<name>.meta` ("key = value" per line, `ParamContainer::Write`,
  src/tools/ParamContainer.cpp:811-832) holding CLASS and the grid (`dims`,
  `N<i>`, `xmin<i>`, `xmax<i>`).  A file sequence appends `_<counter>` to the
  data file name and may share one `.meta` without the counter
  (FileSingle.h:1213-1236, 1377-1394).  A multistate wave function is a
  `WFMultistate` meta with `states = S` plus one file per state named
  `<name>-<i>` (src/qdlib/FileWF.cpp:90-117).
* Stream form (FileSingle.h:141-147, 821-860, 1005-1020): the 16-byte intro
  (the NUL-terminated magic "QDngPrtoBuf" and the version 1 as uint32), then
  per array a uint32 length and a `FileSingleHeader` message
  (src/tools/FileSingleHeader.proto) followed by its payload; a grid wave
  function's payload is a uint32 length, a `GridSystemHeader` message
  (src/qdlib/GridSystem.proto) and the raw data (WFGridSystem::Serialize,
  src/qdlib/WFGridSystem.cpp:140-157).  A multistate stream is a
  `WFMultistate` header with more_files_follow set and no payload, then one
  array per state, more_files_follow set on all but the last
  (FileWF.cpp:119-133).  ZLIB-compressed payloads are read.

The protobuf messages are encoded here directly (varint / 64-bit / length-
delimited fields); no protobuf library is needed.
"""
import os
import struct
import zlib

import numpy as np

from .operators import EIOError, EParamProblem, GridSystem

PBUF_MAGIC = b"QDngPrtoBuf\x00"
PBUF_VERSION = 1
ZLIB_MAGIC = b"ZLIB"   # appended (NUL terminated) to compressed raw files
BZIP_MAGIC = b"BZIP"

WF_CLASSES = ("WFGridCartesian", "WFGridSystem")


# ---------------------------------------------------------------- meta files
def read_meta(path):
    """Key-value pairs of a `.meta` file (comments '#' and blank lines skipped)."""
    meta = {}
    try:
        lines = open(path).read().splitlines()
    except OSError as e:
        raise EIOError(f"Can not read meta file {path}") from e
    for line in lines:
        line = line.strip()
        if not line or line.startswith("#") or "=" not in line:
            continue
        k, v = line.split("=", 1)
        k = k.strip()
        if "[" in k and k.endswith("]"):  # typed keys: key[type] = value
            k = k[:k.index("[")]
        meta[k] = v.strip()
    return meta


def write_meta(path, params):
    with open(path, "w") as f:
        for k, v in params.items():
            f.write(f"{k} = {v}\n")


def grid_params(grid):
    p = {"dims": grid.ndims}
    for i in range(grid.ndims):
        p[f"N{i}"] = grid.n[i]
        p[f"xmin{i}"] = repr(float(grid.xmin[i]))
        p[f"xmax{i}"] = repr(float(grid.xmax[i]))
    return p


def grid_from_meta(meta):
    try:
        dims = int(meta.get("dims", 1))
        n = [int(meta[f"N{i}"]) for i in range(dims)]
        xmin = [float(meta[f"xmin{i}"]) for i in range(dims)]
        xmax = [float(meta[f"xmax{i}"]) for i in range(dims)]
    except KeyError as e:
        raise EParamProblem(f"grid parameter missing in meta data: {e}") from e
    return GridSystem(n, xmin, xmax)


def _data_name(name, suffix, counter=None):
    return f"{name}_{counter}{suffix}" if counter is not None else f"{name}{suffix}"


def _meta_for(name):
    """The meta file of `name`, falling back to the name without a sequence index."""
    p = name + ".meta"
    if os.path.exists(p):
        return read_meta(p)
    if "_" in os.path.basename(name):
        q = name[:name.rfind("_")] + ".meta"
        if os.path.exists(q):
            return read_meta(q)
    raise EIOError(f"Can not read meta file {p}")


def _read_payload(path, nbytes):
    try:
        raw = open(path, "rb").read()
    except OSError as e:
        raise EIOError(f"Can not open binary file for reading {path}") from e
    for magic in (ZLIB_MAGIC, BZIP_MAGIC):
        if raw.endswith(magic + b"\x00"):
            body = raw[:-len(magic) - 1]
            if magic == ZLIB_MAGIC:
                raw = zlib.decompress(body)
            else:
                import bz2
                raw = bz2.decompress(body)
            break
    if len(raw) < nbytes:
        raise EIOError(f"Can not read binary file {path}")
    return raw[:nbytes]


# ------------------------------------------------------------------ raw form
def write_wf(name, psi, grid, nstates=1, suffix=".wf", counter=None):
    """Wave function in the raw form; nstates > 1 writes a WFMultistate."""
    psi = np.ascontiguousarray(psi, dtype="<c16").reshape(-1)
    if psi.size != nstates * grid.npts:
        raise EParamProblem("wave function size does not match grid and states")
    if nstates > 1:
        write_meta(name + ".meta", {"CLASS": "WFMultistate", "states": nstates})
        for i in range(nstates):
            write_wf(f"{name}-{i}", psi[i * grid.npts:(i + 1) * grid.npts], grid, 1, suffix, counter)
        return
    write_meta(name + ".meta", dict(CLASS="WFGridCartesian", **grid_params(grid)))
    psi.tofile(_data_name(name, suffix, counter))


def read_wf(name, suffix=".wf", counter=None):
    """(psi, grid, nstates) of a wave function in the raw form."""
    meta = _meta_for(name if counter is None else f"{name}_{counter}")
    cls = meta.get("CLASS", "")
    if cls == "WFMultistate":
        S = int(meta.get("states", 0))
        if S < 1:
            raise EParamProblem("Init from meta file: Invalid number of states")
        parts, grid = [], None
        for i in range(S):
            p, g, _ = read_wf(f"{name}-{i}", suffix, counter)
            if grid is not None and not g == grid:
                raise EParamProblem("states of a multistate wave function on different grids")
            grid = g
            parts.append(p)
        return np.concatenate(parts), grid, S
    if cls not in WF_CLASSES:
        raise EParamProblem(f"not a grid wave function: CLASS = {cls!r}")
    grid = grid_from_meta(meta)
    raw = _read_payload(_data_name(name, suffix, counter), 16 * grid.npts)
    return np.frombuffer(raw, dtype="<c16").copy(), grid, 1


def write_op(name, values, grid, cls="GridPotential", suffix=".op"):
    """A grid operator (potential, dipole, coupling) in the raw form."""
    v = np.ascontiguousarray(values, dtype="<f8").reshape(-1)
    if v.size != grid.npts:
        raise EParamProblem("operator size does not match the grid")
    write_meta(name + ".meta", dict(CLASS=cls, **grid_params(grid)))
    v.tofile(name + suffix)


def read_op(name, suffix=".op"):
    """(values, grid, CLASS) of a grid operator in the raw form."""
    meta = _meta_for(name)
    grid = grid_from_meta(meta)
    raw = _read_payload(name + suffix, 8 * grid.npts)
    return np.frombuffer(raw, dtype="<f8").copy(), grid, meta.get("CLASS", "")


def write_laser(name, field, dt, suffix=".op"):
    f = np.ascontiguousarray(field, dtype="<f8").reshape(-1)
    write_meta(name + ".meta", {"CLASS": "Laser", "Nt": f.size, "dt": repr(float(dt))})
    f.tofile(name + suffix)


def read_laser(name, suffix=".op"):
    """(field, dt) of a laser field (CLASS = Laser, Nt, dt)."""
    meta = _meta_for(name)
    nt = int(meta["Nt"])
    raw = _read_payload(name + suffix, 8 * nt)
    return np.frombuffer(raw, dtype="<f8").copy(), float(meta["dt"])


# --------------------------------------------------------------- protobuf
def _varint(v):
    out = bytearray()
    v = int(v)
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _key(field, wire):
    return _varint((field << 3) | wire)


def _len_field(field, data):
    return _key(field, 2) + _varint(len(data)) + data


def _decode(buf):
    """Fields of one message: {field: [values]} (varints as int, 64-bit as
    bytes, length-delimited as bytes)."""
    out, i = {}, 0
    while i < len(buf):
        k, i = _read_varint(buf, i)
        field, wire = k >> 3, k & 7
        if wire == 0:
            v, i = _read_varint(buf, i)
        elif wire == 1:
            v, i = buf[i:i + 8], i + 8
        elif wire == 2:
            n, i = _read_varint(buf, i)
            v, i = buf[i:i + n], i + n
        elif wire == 5:
            v, i = buf[i:i + 4], i + 4
        else:
            raise EIOError("Malformated stream: unknown protobuf wire type")
        out.setdefault(field, []).append(v)
    return out


def _read_varint(buf, i):
    shift = v = 0
    while True:
        if i >= len(buf):
            raise EIOError("Malformated stream: truncated varint")
        b = buf[i]
        i += 1
        v |= (b & 0x7F) << shift
        if not b & 0x80:
            return v, i
        shift += 7


def _file_header(cls, name, meta, payload_size, more_files_follow, compression=0):
    """FileSingleHeader (src/tools/FileSingleHeader.proto)."""
    text = "".join(f"{k} = {v}\n" for k, v in meta.items()).encode()
    return (_key(1, 0) + _varint(1 if more_files_follow else 0) + _len_field(2, cls.encode()) +
            _len_field(3, name.encode()) + _len_field(5, text) + _key(6, 0) + _varint(payload_size) +
            _key(7, 0) + _varint(compression))


def _grid_header(grid, data_size):
    """GridSystemHeader (src/qdlib/GridSystem.proto)."""
    msg = _key(1, 0) + _varint(grid.ndims)
    for i in range(grid.ndims):
        dim = (_key(1, 0) + _varint(grid.n[i]) + _key(2, 1) + struct.pack("<d", grid.xmin[i]) +
               _key(3, 1) + struct.pack("<d", grid.xmax[i]))
        msg += _len_field(2, dim)
    return msg + _key(3, 0) + _varint(data_size)


def write_wf_stream(path, psi, grid, nstates=1, compress=False):
    """Wave function in the stream form (one file, all states)."""
    psi = np.ascontiguousarray(psi, dtype="<c16").reshape(-1)
    if psi.size != nstates * grid.npts:
        raise EParamProblem("wave function size does not match grid and states")
    name = os.path.basename(path)
    with open(path, "wb") as f:
        f.write(PBUF_MAGIC + struct.pack("<I", PBUF_VERSION))
        if nstates > 1:
            hdr = _file_header("WFMultistate", name, {"states": nstates}, 0, True)
            f.write(struct.pack("<I", len(hdr)) + hdr)
        for s in range(nstates):
            data = psi[s * grid.npts:(s + 1) * grid.npts].tobytes()
            gh = _grid_header(grid, len(data))
            payload = struct.pack("<I", len(gh)) + gh + data
            if compress:
                payload = zlib.compress(payload)
            hdr = _file_header("WFGridCartesian", name, dict(CLASS="WFGridCartesian", **grid_params(grid)),
                               len(payload), nstates > 1 and s < nstates - 1, 1 if compress else 0)
            f.write(struct.pack("<I", len(hdr)) + hdr + payload)


def read_wf_stream(path):
    """(psi, grid, nstates) of a wave function in the stream form."""
    try:
        buf = open(path, "rb").read()
    except OSError as e:
        raise EIOError(f"Can not open stream {path}") from e
    if buf[:len(PBUF_MAGIC)] != PBUF_MAGIC:
        raise EIOError("Malformated stream. No stream magic found.")
    if struct.unpack_from("<I", buf, 12)[0] != PBUF_VERSION:
        raise EIOError("Wrong stream version")
    i = 16
    parts, grid, more, first = [], None, True, True
    while more and i < len(buf):
        (hl,) = struct.unpack_from("<I", buf, i)
        h = _decode(buf[i + 4:i + 4 + hl])
        i += 4 + hl
        more = bool(h.get(1, [0])[0])
        cls = h.get(2, [b""])[0].decode()
        size = h.get(6, [0])[0]
        comp = h.get(7, [0])[0]
        payload = buf[i:i + size]
        i += size
        if cls == "WFMultistate":
            if not first:
                raise EIOError("nested multistate stream")
            first = False
            continue
        first = False
        if comp != 0:
            payload = zlib.decompress(payload)
        (gl,) = struct.unpack_from("<I", payload, 0)
        g = _decode(payload[4:4 + gl])
        dims = []
        for d in g.get(2, []):
            dd = _decode(d)
            dims.append((dd.get(1, [0])[0], struct.unpack("<d", dd.get(2, [b"\0" * 8])[0])[0],
                         struct.unpack("<d", dd.get(3, [b"\0" * 8])[0])[0]))
        gs = GridSystem([d[0] for d in dims], [d[1] for d in dims], [d[2] for d in dims])
        if grid is not None and not gs == grid:
            raise EParamProblem("states of a multistate wave function on different grids")
        grid = gs
        parts.append(np.frombuffer(payload[4 + gl:4 + gl + 16 * gs.npts], dtype="<c16").copy())
    if not parts:
        raise EIOError("stream holds no wave function")
    return np.concatenate(parts), grid, len(parts)
