"""The library's .dm2p reader (inca_read_dm2p: the read behind inca_load_dm2p, host side) on
generated files, against the reference's format rules (src/mod_intracule.f90:164-195 sniffing,
229-262 batched read) and the oracle's parser of the same bytes.

Cases: flat stream; sequential records with 4-byte markers (same records as the flat file);
8-byte and zero markers (INCA_E_FORMAT); a partial trailing record (dropped); i out of range
or j, k, l below 1 (end of data, as the reference); j, k or l above nprim (an error here, where
the reference reads out of bounds); a broken record marker (end of data); an empty and a missing
file.
"""
import struct

import numpy as np
import pytest

import oracle_lib as O

INCA_E_IO, INCA_E_FORMAT = 3, 4
NPRIM = 27


@pytest.fixture(scope="module")
def reader():
    from inca_parallel_gb300 import build
    build.build()
    from inca_parallel_gb300 import read_dm2p
    return read_dm2p


def _records(n=200, seed=3):
    rng = np.random.default_rng(seed)
    ijkl = rng.integers(1, NPRIM + 1, size=(n, 4)).astype(np.int32)
    v = rng.normal(size=n)
    return ijkl, v


def _flat(ijkl, v):
    return b"".join(struct.pack("<4id", *map(int, q), float(x)) for q, x in zip(ijkl, v))


def _sequential(ijkl, v, marker=24, fmt="<i"):
    m = struct.pack(fmt, marker)
    return b"".join(m + struct.pack("<4id", *map(int, q), float(x)) + m for q, x in zip(ijkl, v))


def _write(tmp_path, name, raw):
    p = tmp_path / name
    p.write_bytes(raw)
    return str(p)


def _check(reader, path, raw, n_expected):
    ijkl, v = reader(path, NPRIM)
    assert len(v) == n_expected
    oi, ov = O.parse_dm2p_bytes(raw, NPRIM)
    np.testing.assert_array_equal(ijkl, oi)
    np.testing.assert_array_equal(v, ov)
    return ijkl, v


def test_flat_and_sequential_agree(reader, tmp_path):
    q, v = _records()
    raw_f, raw_s = _flat(q, v), _sequential(q, v)
    fi, fv = _check(reader, _write(tmp_path, "flat.dm2p", raw_f), raw_f, len(v))
    si, sv = _check(reader, _write(tmp_path, "seq.dm2p", raw_s), raw_s, len(v))
    np.testing.assert_array_equal(fi, q)
    np.testing.assert_array_equal(si, fi)
    np.testing.assert_array_equal(sv, fv)


def test_reference_fixture(reader, tmp_path, ch4):
    raw = ch4["raw"]
    _check(reader, _write(tmp_path, "ch4.dm2p", raw), raw, 142884)


@pytest.mark.parametrize("kind", ["8-byte", "zero"])
def test_marker_formats_rejected(reader, tmp_path, kind):
    from inca_parallel_gb300 import IncaError
    q, v = _records(10)
    raw = _sequential(q, v, 24, "<q") if kind == "8-byte" else _sequential(q, v, 0)
    with pytest.raises(IncaError) as e:
        reader(_write(tmp_path, kind + ".dm2p", raw), NPRIM)
    assert e.value.code == INCA_E_FORMAT
    with pytest.raises(ValueError):
        O.parse_dm2p_bytes(raw, NPRIM)


def test_partial_trailing_record(reader, tmp_path):
    q, v = _records(50)
    raw = _flat(q, v) + b"\x01" * 10
    _check(reader, _write(tmp_path, "trail.dm2p", raw), raw, 50)
    raw = _sequential(q, v)[:-7]
    _check(reader, _write(tmp_path, "trail_seq.dm2p", raw), raw, 49)


@pytest.mark.parametrize("col,val", [(0, NPRIM + 1), (0, 0), (1, 0), (2, -3), (3, 0)])
def test_index_out_of_range_ends_the_data(reader, tmp_path, col, val):
    q, v = _records(40)
    q[17, col] = val
    for name, raw in (("f", _flat(q, v)), ("s", _sequential(q, v))):
        _check(reader, _write(tmp_path, f"oor_{name}.dm2p", raw), raw, 17)


@pytest.mark.parametrize("col", [1, 2, 3])
def test_index_above_nprim_is_an_error(reader, tmp_path, col):
    from inca_parallel_gb300 import IncaError
    q, v = _records(40)
    q[9, col] = NPRIM + 5
    with pytest.raises(IncaError) as e:
        reader(_write(tmp_path, "above.dm2p", _flat(q, v)), NPRIM)
    assert e.value.code == INCA_E_FORMAT and "record 10" in str(e.value)


def test_broken_marker_ends_the_data(reader, tmp_path):
    q, v = _records(30)
    raw = bytearray(_sequential(q, v))
    raw[12 * 32 + 28:12 * 32 + 32] = struct.pack("<i", 20)  # trailing marker of record 13
    ijkl, vv = reader(_write(tmp_path, "marker.dm2p", bytes(raw)), NPRIM)
    assert len(vv) == 12
    np.testing.assert_array_equal(ijkl, q[:12])


def test_empty_and_missing(reader, tmp_path):
    from inca_parallel_gb300 import IncaError
    ijkl, v = reader(_write(tmp_path, "empty.dm2p", b""), NPRIM)
    assert len(v) == 0 and ijkl.shape == (0, 4)
    with pytest.raises(IncaError) as e:
        reader(str(tmp_path / "nope.dm2p"), NPRIM)
    assert e.value.code == INCA_E_IO
