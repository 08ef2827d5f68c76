"""Seismic Unix trace files (fwi_su_*): the C++ reader and writer against an
independent byte-level layout written here with struct (240-byte header:
tracl int32 at byte 0, ns uint16 at 114, dt uint16 in microseconds at 116;
then ns float32 samples), in both byte orders."""
import struct

import numpy as np
import pytest


def _write_su_py(path, data, dt_us, big):
    e = ">" if big else "<"
    nt, ntr = data.shape
    with open(path, "wb") as f:
        for j in range(ntr):
            h = bytearray(240)
            struct.pack_into(e + "i", h, 0, j + 1)
            struct.pack_into(e + "H", h, 114, nt)
            struct.pack_into(e + "H", h, 116, dt_us)
            struct.pack_into(e + "i", h, 4, 777)        # other header words are not data
            f.write(bytes(h))
            f.write(np.asarray(data[:, j], dtype=e + "f4").tobytes())


@pytest.mark.parametrize("big", [False, True])
def test_su_read_matches_layout(tmp_path, big):
    import fwi_gb300 as F
    rng = np.random.default_rng(1)
    data = rng.standard_normal((123, 7)).astype(np.float32)
    p = tmp_path / "shot.su"
    _write_su_py(p, data, 2000, big)
    ns, dt, ntr = F.su_info(p, big_endian=big)
    assert (ns, ntr) == (123, 7) and dt == np.float32(2000e-6)
    assert np.array_equal(F.su_read(p, 123, 7, big_endian=big), data)
    assert np.array_equal(F.su_read(p, 123, 3, big_endian=big), data[:, :3])    # the first traces only
    with pytest.raises(F.FwiError):
        F.su_read(p, 123, 8, big_endian=big)                                    # past the end of the file


@pytest.mark.parametrize("big", [False, True])
def test_su_write_headers_and_round_trip(tmp_path, big):
    import fwi_gb300 as F
    rng = np.random.default_rng(2)
    data = rng.standard_normal((301, 5)).astype(np.float32)
    p = tmp_path / "new.su"
    F.su_write(p, data, 0.0025, big_endian=big)
    raw = p.read_bytes()
    e = ">" if big else "<"
    assert len(raw) == 5 * (240 + 4 * 301)
    for j in range(5):
        h = raw[j * (240 + 1204): j * (240 + 1204) + 240]
        assert struct.unpack_from(e + "i", h, 0)[0] == j + 1          # tracl
        assert struct.unpack_from(e + "i", h, 4)[0] == j + 1          # tracr
        assert struct.unpack_from(e + "H", h, 28)[0] == 1             # trid: live trace
        assert struct.unpack_from(e + "H", h, 114)[0] == 301
        assert struct.unpack_from(e + "H", h, 116)[0] == int(np.float32(0.0025) * np.float32(1e6))
        body = np.frombuffer(raw, dtype=e + "f4", count=301, offset=j * (240 + 1204) + 240)
        assert np.array_equal(body, data[:, j])
    assert np.array_equal(F.su_read(p, 301, 5, big_endian=big), data)


def test_read_nav(tmp_path):
    import fwi_gb300 as F
    p = tmp_path / "nav.txt"
    p.write_text("101 6250.0 500.5\n102, 6500.25, 498.0\n\n  103\t6750.5   -497.75\n")
    ids, xs, bat = F.read_nav(p)
    assert ids.tolist() == [101, 102, 103]
    assert xs.tolist() == [6250.0, 6500.25, 6750.5] and bat.tolist() == [500.5, 498.0, -497.75]
    (tmp_path / "bad.txt").write_text("101 6250.0\n")
    with pytest.raises(F.FwiError):
        F.read_nav(tmp_path / "bad.txt")


@pytest.mark.parametrize("big", [False, True])
def test_supershot_sum_of_coded_obs_files(tmp_path, big):
    """get_obs_data (get_was_data.f90:241-288): the first traces of each OBS
    file summed with their coding factors, in FP32 and in file order."""
    import fwi_gb300 as F
    rng = np.random.default_rng(5)
    nt, ntr = 90, 6
    gathers = [rng.standard_normal((nt, ntr + 2)).astype(np.float32) for _ in range(3)]
    paths = []
    for k, g in enumerate(gathers):
        p = tmp_path / f"OBS{k + 1}.su"
        _write_su_py(p, g, 4000, big)
        paths.append(p)
    coding = np.array([1.0, -1.0, 0.5], np.float32)
    got = F.su_supershot(paths, coding, nt, ntr, big_endian=big)
    ref = np.zeros((nt, ntr), np.float32)
    for c, g in zip(coding, gathers):
        ref = (ref + c * g[:, :ntr]).astype(np.float32)
    assert np.array_equal(got, ref)
    with pytest.raises(F.FwiError):
        F.su_supershot(paths, coding, nt, ntr + 3, big_endian=big)


def test_read_nav_obs_and_was_shot_lists(tmp_path):
    """read_nav_obs / read_nav_shot_was lists: OBS number, x, depth."""
    import fwi_gb300 as F
    p = tmp_path / "nav_obs.txt"
    p.write_text("1 2500.0 -2801.5\n2,7500.0,2790.25\n")
    ids, xs, zs = F.read_nav(p)
    assert ids.tolist() == [1, 2] and xs.tolist() == [2500.0, 7500.0] and zs.tolist() == [-2801.5, 2790.25]
