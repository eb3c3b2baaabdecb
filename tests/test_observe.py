"""Host logic of the observables and the orientation scan (no GPU): the PNG
writer, the phase colour table, slice-index resolution, the growth-rate fit
and the anisotropy index, each against an independent computation."""
import math
import struct
import zlib

import numpy as np
import pytest


def read_png(path):
    """Minimal decoder for the 8-bit RGB, filter-0 PNGs write_png produces."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(tag + body) & 0xFFFFFFFF
        chunks.setdefault(tag, b"")
        chunks[tag] += body
        pos += 12 + n
    w, h, depth, ctype, _, _, _ = struct.unpack(">IIBBBBB", chunks[b"IHDR"])
    assert (depth, ctype) == (8, 2)
    raw = zlib.decompress(chunks[b"IDAT"])
    rows = [raw[r * (3 * w + 1):(r + 1) * (3 * w + 1)] for r in range(h)]
    assert all(row[0] == 0 for row in rows)
    return np.frombuffer(b"".join(row[1:] for row in rows), np.uint8).reshape(h, w, 3)


def test_png_round_trip(tmp_path):
    from mpf3d.observe import write_png
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (7, 11, 3), dtype=np.uint8)
    p = tmp_path / "a.png"
    write_png(str(p), img)
    assert np.array_equal(read_png(str(p)), img)


def test_phase_colours_follow_tab20_scaling():
    """imshow(cmap="tab20", vmin=0, vmax=N-1): value v -> colour int(v/(N-1)*20), capped at 19."""
    from mpf3d.observe import TAB20, phase_colours
    N = 9
    ids = np.arange(N)
    got = phase_colours(ids, N)
    want = TAB20[[min(int(v / (N - 1) * 20), 19) for v in ids]]
    assert np.array_equal(got, want)
    assert np.array_equal(phase_colours([0, 1], 1), TAB20[[0, 19]])  # vmax floors at 1


def test_phase_map_png_orientation(tmp_path):
    """First slice axis to the right, second axis upwards (origin="lower")."""
    from mpf3d.observe import TAB20, save_phase_map_png
    ids = np.zeros((4, 3), np.int32)
    ids[3, 0] = 1  # x = 3, y = 0: bottom-right pixel
    p = tmp_path / "m.png"
    save_phase_map_png(str(p), {"ids": ids}, 2)
    img = read_png(str(p))
    assert img.shape == (3, 4, 3)
    assert np.array_equal(img[2, 3], TAB20[19]) and np.array_equal(img[0, 0], TAB20[0])


@pytest.mark.parametrize("axis,index,want", [("xy", None, 5), ("xz", None, 4), ("yz", None, 3),
                                             ("xy", 99, 9), ("yz", -4, 0)])
def test_slice_index_resolution(axis, index, want):
    from mpf3d.observe import resolve_slice_index
    assert resolve_slice_index(axis, (7, 8, 10), index) == want


def test_growth_rate_fit_trailing_fraction_and_cutoff():
    from mpf3d.scan import fit_growth_rate
    t = np.arange(11) * 5e-4
    r = np.where(t < 2e-3, 1e-3 + 0.1 * t, 1e-3 + 0.1 * 2e-3 + 0.3 * (t - 2e-3))
    ts = [{"time": a, "equivalent_radius": b} for a, b in zip(t, r)]
    rate, i0, i1, n = fit_growth_rate(ts, 0.5)
    assert (i0, i1, n) == (5, 10, 6)
    assert rate == pytest.approx(0.3, rel=1e-9)
    rate, i0, i1, n = fit_growth_rate(ts, 0.5, fit_end_time_s=1.5e-3)
    assert (i0, i1, n) == (0, 3, 4)
    assert rate == pytest.approx(0.1, rel=1e-9)
    ts[-1]["equivalent_radius"] = float("nan")
    assert fit_growth_rate(ts, 0.5)[3] == 5
    assert math.isnan(fit_growth_rate(ts[:1], 0.5)[0])


def test_anisotropy_index_and_modes():
    from mpf3d.scan import anisotropy_index, resolve_anisotropy_mode
    row = {"radius_x": 2.0, "radius_y": 4.0, "radius_z": float("nan"), "radius_diag111": 3.0}
    assert anisotropy_index(row) == pytest.approx((4.0 - 2.0) / 3.0)
    assert math.isnan(anisotropy_index({"radius_x": 1.0}))
    assert resolve_anisotropy_mode("full", 0.36, 0.05) == (1, 1, 0.36, 0.05)
    assert resolve_anisotropy_mode("isotropic", 0.36, 0.05) == (0, 0, 0.0, 1.0)
    assert resolve_anisotropy_mode("energetic_only", 0.36, 0.05) == (1, 1, 0.36, 1.0)
    assert resolve_anisotropy_mode("kinetic_only", 0.36, 0.05) == (1, 0, 0.0, 0.05)
    with pytest.raises(ValueError):
        resolve_anisotropy_mode("other", 0.36, 0.05)


def test_default_orientation_cases():
    pytest.importorskip("scipy")
    from mpf3d.scan import resolve_orientation_cases
    cs = resolve_orientation_cases()
    assert [c["label"] for c in cs] == ["{100}", "{110}", "{111}", "mid1", "mid2"]
    q111 = np.array(cs[2]["quaternion"])
    from scipy.spatial.transform import Rotation
    v = Rotation.from_quat(q111).apply(np.array([1.0, 1.0, 1.0]) / math.sqrt(3.0))
    assert np.allclose(v, [0, 0, 1], atol=1e-12)
    assert np.allclose(cs[1]["euler_deg"], [0.0, 45.0, 0.0], atol=1e-9)
