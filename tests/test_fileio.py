"""QDng file formats (raw + .meta, protobuf stream, multistate naming)."""
import struct

import numpy as np
import pytest

from qdng_gb300 import fileio
from qdng_gb300 import operators as op


def _psi(n, seed=0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def test_meta_parsing_matches_qdng_text(tmp_path):
    p = tmp_path / "pot.meta"
    p.write_text("# Generated file\n# comment\nCLASS = GridPotential \ndims = 1 \nN0 = 128\n"
                 "xmin0 = 1.8897\nxmax0 = 6.1104\nmass[double] = 1763.2\n\n")
    m = fileio.read_meta(str(p))
    assert m["CLASS"] == "GridPotential" and m["N0"] == "128" and m["mass"] == "1763.2"
    g = fileio.grid_from_meta(m)
    assert g.n == [128] and g.xmin == [1.8897] and g.xmax == [6.1104]


def test_raw_wf_and_op_round_trip(tmp_path, fixtures):
    g = op.GridSystem([32, 24], [-4.0, -3.0], [4.0, 3.5])
    psi = _psi(g.npts)
    fileio.write_wf(str(tmp_path / "psi"), psi, g)
    assert (tmp_path / "psi.wf").stat().st_size == 16 * g.npts
    meta = fileio.read_meta(str(tmp_path / "psi.meta"))
    assert meta["CLASS"] == "WFGridCartesian" and meta["N1"] == "24"
    back, g2, S = fileio.read_wf(str(tmp_path / "psi"))
    assert S == 1 and g2 == g and np.array_equal(back, psi)
    n, xmin, xmax = fixtures["GridPot0_grid"]
    g1 = op.GridSystem([int(n)], [xmin], [xmax])
    fileio.write_op(str(tmp_path / "GridPot0"), fixtures["GridPot0"], g1)
    v, g3, cls = fileio.read_op(str(tmp_path / "GridPot0"))
    assert cls == "GridPotential" and g3 == g1 and np.array_equal(v, fixtures["GridPot0"])
    raw = open(tmp_path / "GridPot0.op", "rb").read()
    assert raw == np.asarray(fixtures["GridPot0"], dtype="<f8").tobytes()  # plain little-endian doubles


def test_multistate_raw_naming(tmp_path):
    g = op.GridSystem([16], [0.0], [1.0])
    psi = _psi(3 * g.npts, 1)
    fileio.write_wf(str(tmp_path / "ms"), psi, g, nstates=3)
    assert fileio.read_meta(str(tmp_path / "ms.meta")) == {"CLASS": "WFMultistate", "states": "3"}
    for i in range(3):
        assert (tmp_path / f"ms-{i}.wf").exists() and (tmp_path / f"ms-{i}.meta").exists()
    back, g2, S = fileio.read_wf(str(tmp_path / "ms"))
    assert S == 3 and g2 == g and np.array_equal(back, psi)


def test_sequence_and_compressed_raw(tmp_path):
    g = op.GridSystem([8], [0.0], [1.0])
    psi = _psi(8, 2)
    fileio.write_wf(str(tmp_path / "seq"), psi, g, counter=5)
    assert (tmp_path / "seq_5.wf").exists()
    back, _, _ = fileio.read_wf(str(tmp_path / "seq"), counter=5)
    assert np.array_equal(back, psi)
    # zlib payload with the trailing magic of a compressed raw file
    import zlib
    (tmp_path / "z.wf").write_bytes(zlib.compress(psi.astype("<c16").tobytes()) + b"ZLIB\x00")
    fileio.write_meta(str(tmp_path / "z.meta"), dict(CLASS="WFGridCartesian", **fileio.grid_params(g)))
    back, _, _ = fileio.read_wf(str(tmp_path / "z"))
    assert np.array_equal(back, psi)


@pytest.mark.parametrize("nstates,compress", [(1, False), (2, False), (3, True)])
def test_stream_round_trip(tmp_path, nstates, compress):
    g = op.GridSystem([12, 10], [-1.0, -2.0], [1.0, 2.0])
    psi = _psi(nstates * g.npts, 3)
    path = str(tmp_path / "psi.wf")
    fileio.write_wf_stream(path, psi, g, nstates, compress)
    buf = open(path, "rb").read()
    assert buf[:16] == b"QDngPrtoBuf\x00" + struct.pack("<I", 1)
    back, g2, S = fileio.read_wf_stream(path)
    assert S == nstates and g2 == g and np.array_equal(back, psi)


def test_stream_header_encoding(tmp_path):
    """Field layout of the first FileSingleHeader: more_files_follow (1,
    varint), class (2, bytes), ..., payload_size (6), compression (7)."""
    g = op.GridSystem([4], [0.0], [1.0])
    path = str(tmp_path / "a.wf")
    fileio.write_wf_stream(path, np.ones(4, dtype=complex), g)
    buf = open(path, "rb").read()
    (hl,) = struct.unpack_from("<I", buf, 16)
    h = fileio._decode(buf[20:20 + hl])
    assert h[1] == [0] and h[2] == [b"WFGridCartesian"] and h[7] == [0]
    payload = buf[20 + hl:20 + hl + h[6][0]]
    (gl,) = struct.unpack_from("<I", payload, 0)
    gh = fileio._decode(payload[4:4 + gl])
    assert gh[1] == [1] and gh[3] == [64]
    d = fileio._decode(gh[2][0])
    assert d[1] == [4] and struct.unpack("<d", d[3][0])[0] == 1.0


def test_errors(tmp_path):
    with pytest.raises(op.EIOError):
        fileio.read_wf(str(tmp_path / "missing"))
    (tmp_path / "bad.wf").write_bytes(b"nonsense" * 4)
    with pytest.raises(op.EIOError):
        fileio.read_wf_stream(str(tmp_path / "bad.wf"))
    g = op.GridSystem([8], [0.0], [1.0])
    with pytest.raises(op.EParamProblem):
        fileio.write_wf(str(tmp_path / "x"), np.ones(7, dtype=complex), g)
