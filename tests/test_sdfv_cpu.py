"""`.sdfv` volume ingest and writer in the C ABI (mm3e_volume_parse_sdfv / mm3e_volume_write_sdfv)
against mm3e-kit/src/volume.rs:115-248 and its test (mm3e-kit/tests/kit.rs:264-295). Host-only
entry points: no GPU is needed."""
import struct

import numpy as np
import pytest

from mm3e_cuda.scene import SdfVolume
from mm3e_cuda.scene_io import SceneFormatError, parse_sdfv, serialize_sdfv

HEADER = 44


def _vol():
    return SdfVolume((2, 2, 2), (-1.0, -2.0, -3.0), (0.5, 0.75, 1.25), [0.0, 0.5, 1.0, 1.5, -0.25, 0.25, 0.75, 1.25])


def _raw(dims, vmin, cell, data):
    return b"MM3ESDF1" + struct.pack("<3I", *dims) + struct.pack("<6f", *vmin, *cell) + struct.pack(
        f"<{len(data)}f", *data)


def test_roundtrip_and_layout(tmp_path):
    """kit.rs:264-295: magic, exact round trip, truncation and magic rejections, file round trip."""
    vol = _vol()
    b = serialize_sdfv(vol)
    assert b[:8] == b"MM3ESDF1"
    assert b == _raw(vol.dims, vol.min, vol.cell, list(vol.data))  # little-endian u32 / f32 fields
    r = parse_sdfv(b)
    assert r.dims == vol.dims and r.min == vol.min and r.cell == vol.cell
    assert np.array_equal(r.data, vol.data)
    with pytest.raises(SceneFormatError, match="shorter than the header"):
        parse_sdfv(b[:12])
    with pytest.raises(SceneFormatError, match="magic/version mismatch"):
        parse_sdfv(b"X" + b[1:])
    path = tmp_path / "v.sdfv"
    path.write_bytes(vol.to_sdfv_bytes())
    assert np.array_equal(SdfVolume.from_sdfv_bytes(path.read_bytes()).data, vol.data)


def test_larger_volume_bit_exact():
    rng = np.random.default_rng(7)
    data = rng.standard_normal(5 * 3 * 4).astype(np.float32)
    data[3] = -0.0
    data[4] = np.float32(1e-45)  # subnormal survives
    vol = SdfVolume((5, 3, 4), (0.1, -0.2, 0.3), (0.01, 0.02, 0.03), data)
    r = parse_sdfv(serialize_sdfv(vol))
    assert r.dims == (5, 3, 4)
    assert r.data.view(np.uint32).tolist() == data.view(np.uint32).tolist()


@pytest.mark.parametrize("mutate, message", [
    (lambda: _raw((2, 2, 2), (float("nan"), 0, 0), (1, 1, 1), [0.0] * 8), "non-finite f32 while reading min.x"),
    (lambda: _raw((2, 2, 2), (0, 0, 0), (1, float("inf"), 1), [0.0] * 8), "non-finite f32 while reading cell.y"),
    (lambda: _raw((2, 2, 2), (0, 0, 0), (1, 1, 1), [0.0] * 7), "byte length 72 does not match expected 76"),
    (lambda: _raw((2, 2, 2), (0, 0, 0), (1, 1, 1), [0.0] * 9), "byte length 80 does not match expected 76"),
    (lambda: _raw((2, 2, 2), (0, 0, 0), (1, 1, 1), [0.0] * 5 + [float("nan")] + [0.0] * 2),
     "non-finite f32 while reading sample 5"),
    (lambda: _raw((1, 2, 2), (0, 0, 0), (1, 1, 1), [0.0] * 4), "dims must all be >= 2"),
    (lambda: _raw((2, 2, 2), (0, 0, 0), (1, 0, 1), [0.0] * 8), "cell sizes must be positive and finite"),
    (lambda: _raw((2, 2, 2), (0, 0, 0), (1, 1, -1), [0.0] * 8), "cell sizes must be positive and finite"),
    (lambda: _raw((0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF), (0, 0, 0), (1, 1, 1), []), "dimensions overflow"),
    (lambda: _raw((0xFFFFFFFF, 0xFFFFFFFF, 1), (0, 0, 0), (1, 1, 1), []), "payload length overflows"),
    (lambda: _raw((0, 2, 2), (0, 0, 0), (1, 1, 1), []), "dims must all be >= 2"),
])
def test_parse_rejections(mutate, message):
    """from_sdfv_bytes's error order (volume.rs:140-176): header fields, overflow, byte length,
    each sample, then SdfVolume::new's layout rules."""
    with pytest.raises(SceneFormatError, match=message):
        parse_sdfv(mutate())


def test_writer_validates():
    """to_sdfv_bytes validates first (volume.rs:119-121)."""
    bad = SdfVolume((2, 2, 2), (0, 0, 0), (1, 1, 1), [0.0] * 3 + [float("inf")] + [0.0] * 4)
    with pytest.raises(SceneFormatError, match="SdfVolume sample 3 is non-finite"):
        serialize_sdfv(bad)
    with pytest.raises(SceneFormatError, match="dims must all be >= 2"):
        serialize_sdfv(SdfVolume((2, 1, 2), (0, 0, 0), (1, 1, 1), [0.0] * 4))
    with pytest.raises(SceneFormatError, match="min must be finite"):
        serialize_sdfv(SdfVolume((2, 2, 2), (0, float("nan"), 0), (1, 1, 1), [0.0] * 8))
    assert len(serialize_sdfv(_vol())) == HEADER + 8 * 4
