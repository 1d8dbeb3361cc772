"""Binary star catalogues and parameter files: round trips against the
reference-format text files, the mapped view, and rejection of malformed
files (no GPU)."""
import os
import struct

import numpy as np
import pytest

from conftest import golden_cases, load_case


def test_catalogue_round_trip(built_library, tmp_path):
    import milkywayathome_client_gb300 as mw
    for name in ("basic_1stream", "ragged_sizes", "single_cell_single_star"):
        _, sf, _ = load_case(name)
        sp = mw.StarPoints.read(sf)
        p = str(tmp_path / f"{name}.mwsb")
        sp.write_binary(p)
        back = mw.StarPoints.read_binary(p)
        assert np.array_equal(back.to_array(), sp.to_array())
        with mw.StarCatalogue(p) as cat:
            a = sp.to_array()
            assert cat.number_stars == a.shape[0]
            assert np.array_equal(cat.l, a[:, 0]) and np.array_equal(cat.b, a[:, 1]) and np.array_equal(cat.r, a[:, 2])
            for col in (cat.l, cat.b, cat.r):
                assert col.ctypes.data % 64 == 0


def test_catalogue_layout(built_library, tmp_path):
    import milkywayathome_client_gb300 as mw
    a = np.array([[10.0, 20.0, 30.0], [11.0, 21.0, 31.0], [12.0, 22.0, 32.0]])
    p = str(tmp_path / "c.mwsb")
    mw.StarCatalogue.write(p, a)
    raw = open(p, "rb").read()
    magic, ver, hb, n, ol, ob, orr, fb, res = struct.unpack("<8sIIQQQQQQ", raw[:64])
    assert (magic, ver, hb, n, res) == (b"MWSEPCAT", 1, 64, 3, 0)
    assert (ol, ob, orr) == (64, 128, 192) and fb == len(raw) == 192 + 24
    assert struct.unpack("<3d", raw[ob:ob + 24]) == (20.0, 21.0, 22.0)


def test_empty_catalogue(built_library, tmp_path):
    import milkywayathome_client_gb300 as mw
    p = str(tmp_path / "empty.mwsb")
    mw.StarCatalogue.write(p, np.zeros((0, 3)))
    with mw.StarCatalogue(p) as cat:
        assert cat.number_stars == 0
    assert mw.StarPoints.read_binary(p).number_stars == 0


def _corrupt(src, dst, at, data):
    raw = bytearray(open(src, "rb").read())
    raw[at:at + len(data)] = data
    open(dst, "wb").write(bytes(raw))


def test_malformed_catalogues_are_rejected(built_library, tmp_path):
    import milkywayathome_client_gb300 as mw
    good = str(tmp_path / "good.mwsb")
    mw.StarCatalogue.write(good, np.arange(30, dtype=float).reshape(10, 3))
    bad = str(tmp_path / "bad.mwsb")
    cases = [(0, b"MWSEPCAX"), (8, struct.pack("<I", 2)), (16, struct.pack("<Q", 11)),
             (24, struct.pack("<Q", 2 ** 64 - 8)), (40, struct.pack("<Q", 190)), (48, struct.pack("<Q", 1000))]
    for at, data in cases:
        _corrupt(good, bad, at, data)
        with pytest.raises(mw.MwsepError):
            mw.StarCatalogue(bad)
        with pytest.raises(mw.MwsepError):
            mw.StarPoints.read_binary(bad)
    raw = open(good, "rb").read()
    open(bad, "wb").write(raw[:-8])
    with pytest.raises(mw.MwsepError):
        mw.StarCatalogue(bad)
    open(bad, "wb").write(raw[:40])
    with pytest.raises(mw.MwsepError):
        mw.StarCatalogue(bad)
    with pytest.raises(mw.MwsepError):
        mw.StarCatalogue(str(tmp_path / "missing.mwsb"))


def _fields(ap):
    s = ap.struct
    out = {k: getattr(s, k) for k in ("parameters_version", "number_background_parameters", "background_weight",
                                      "number_streams", "number_stream_parameters", "convolve", "sgr_coordinates",
                                      "aux_bg_profile", "wedge", "number_integrals")}
    nb, S, P = s.number_background_parameters, s.number_streams, s.number_stream_parameters
    for k in ("background_parameters", "background_step", "background_min", "background_max",
              "background_optimize"):
        out[k] = [getattr(s, k)[i] for i in range(nb)]
    for k in ("stream_weights", "stream_weight_step", "stream_weight_min", "stream_weight_max",
              "stream_weight_optimize"):
        out[k] = [getattr(s, k)[i] for i in range(S)]
    for k in ("stream_parameters", "stream_step", "stream_min", "stream_max", "stream_optimize"):
        out[k] = [[getattr(s, k)[i][j] for j in range(P)] for i in range(S)]
    out["integral"] = [ap.area(i) for i in range(s.number_integrals)]
    return out


@pytest.mark.parametrize("name", golden_cases())
def test_parameter_round_trip(built_library, tmp_path, name):
    import milkywayathome_client_gb300 as mw
    pf, _, _ = load_case(name)
    ap = mw.AstronomyParameters.read(pf)
    p = str(tmp_path / "p.mwsp")
    ap.write_binary(p)
    back = mw.AstronomyParameters.read_binary(p)
    assert _fields(back) == _fields(ap)
    t1, t2 = str(tmp_path / "a.txt"), str(tmp_path / "b.txt")
    ap.write(t1)
    back.write(t2)
    assert open(t1).read() == open(t2).read()


def test_corrupt_parameter_file_is_rejected(built_library, tmp_path):
    import milkywayathome_client_gb300 as mw
    pf, _, _ = load_case("three_streams")
    p = str(tmp_path / "p.mwsp")
    mw.AstronomyParameters.read(pf).write_binary(p)
    raw = bytearray(open(p, "rb").read())
    bad = str(tmp_path / "bad.mwsp")
    for at in (0, 9, 20, len(raw) // 2, len(raw) - 3):
        r = bytearray(raw)
        r[at] ^= 0x40
        open(bad, "wb").write(bytes(r))
        with pytest.raises(mw.MwsepError):
            mw.AstronomyParameters.read_binary(bad)
    open(bad, "wb").write(bytes(raw[:-9]))
    with pytest.raises(mw.MwsepError):
        mw.AstronomyParameters.read_binary(bad)


def _fnv1a(data):
    h = 1469598103934665603
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_parameter_format_1_still_loads(built_library, tmp_path):
    """Format 1 stored number_background_parameters values of each background
    array and no separate count; a file in it (the format-2 file of a problem
    without the aux quirk, its count removed) still loads to the same struct."""
    import struct
    import milkywayathome_client_gb300 as mw
    pf, _, _ = load_case("aux_profile")
    ap = mw.AstronomyParameters.read(pf)
    p2 = str(tmp_path / "p2.mwsp")
    ap.write_binary(p2)
    raw = open(p2, "rb").read()
    magic, version, body_len = raw[:8], struct.unpack("<I", raw[8:12])[0], struct.unpack("<I", raw[12:16])[0]
    assert version == 2
    body = raw[16:16 + body_len]
    nb, nv = struct.unpack("<ii", body[8:16])
    assert nb == nv
    body1 = body[:12] + body[16:]  # drop the stored count after number_background_parameters
    p1 = str(tmp_path / "p1.mwsp")
    with open(p1, "wb") as f:
        f.write(magic + struct.pack("<II", 1, len(body1)) + body1 + struct.pack("<Q", _fnv1a(body1)))
    back = mw.AstronomyParameters.read_binary(p1)
    assert _fields(back) == _fields(ap)
