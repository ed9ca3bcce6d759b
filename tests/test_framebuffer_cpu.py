"""Framebuffer encoders of the host mirror (mm3e_cuda.to_rgba8 / to_u32 / to_bmp) against known
answers worked out from mm3e-kit/src/framebuffer.rs:54-127: straight alpha over a background,
the u8 quantisation (clamp * 255 + 0.5, truncated), the 0x00RRGGBB packing and the 24-bit
bottom-up BMP layout."""
import numpy as np

import mm3e_cuda

BG = (0.2, 0.4, 0.6, 1.0)


def _frame():
    """3 x 2 RGBA f32 pixels covering opaque, transparent, over-range, negative, NaN and alpha > 1."""
    nan = float("nan")
    return np.array([[[1.0, 0.5, 0.0, 1.0], [0.0, 0.0, 0.0, 0.0], [2.0, -1.0, nan, 0.5]],
                     [[0.25, 0.25, 0.25, 2.0], [0.1, 0.9, 0.3, 1.0], [1.0, 1.0, 1.0, -1.0]]], np.float32)


# Per pixel over BG: (1, .5, 0, a=1) -> 255 128 0; (a=0) -> BG = 51 102 153; (2, -1, NaN, a=.5)
# -> r = 1 + .1 = 1.1 -> 255, g = -.5 + .2 = -.3 -> 0, b NaN -> 0; (.25, a=2 -> 1) -> 64 64 64;
# (.1, .9, .3) -> 26 230 77; (a=-1 -> 0) -> BG.
RGB = np.array([[[255, 128, 0], [51, 102, 153], [255, 0, 0]],
                [[64, 64, 64], [26, 230, 77], [51, 102, 153]]], np.uint8)


def test_to_rgba8_known_answers():
    out = mm3e_cuda.to_rgba8(_frame(), BG)
    assert out.shape == (2, 3, 4) and out.dtype == np.uint8
    assert np.array_equal(out[..., :3], RGB)
    assert (out[..., 3] == 255).all()
    black = mm3e_cuda.to_rgba8(_frame())  # the default background is black
    assert tuple(black[0, 1, :3]) == (0, 0, 0) and tuple(black[0, 0, :3]) == (255, 128, 0)


def test_to_u32_packs_rrggbb():
    out = mm3e_cuda.to_u32(_frame(), BG)
    assert out.dtype == np.uint32 and out.shape == (2, 3)
    want = (RGB[..., 0].astype(np.uint32) << 16) | (RGB[..., 1].astype(np.uint32) << 8) | RGB[..., 2]
    assert np.array_equal(out, want)
    assert out[0, 0] == 0x00FF8000


def test_to_bmp_layout():
    bmp = mm3e_cuda.to_bmp(_frame(), BG)
    row_bytes = 3 * 3 + 3  # 9 bytes of pixels padded to 12
    assert len(bmp) == 54 + 2 * row_bytes
    le = lambda off, n, signed=False: int.from_bytes(bmp[off:off + n], "little", signed=signed)
    assert bmp[:2] == b"BM" and le(2, 4) == len(bmp) and le(6, 4) == 0 and le(10, 4) == 54
    assert le(14, 4) == 40 and le(18, 4, True) == 3 and le(22, 4, True) == 2
    assert le(26, 2) == 1 and le(28, 2) == 24 and le(30, 4) == 0 and le(34, 4) == 2 * row_bytes
    assert le(38, 4, True) == 2835 and le(42, 4, True) == 2835 and le(46, 4) == 0 and le(50, 4) == 0
    rows = np.frombuffer(bmp[54:], np.uint8).reshape(2, row_bytes)
    assert np.array_equal(rows[0, :9].reshape(3, 3), RGB[1, :, ::-1])  # bottom row first, BGR
    assert np.array_equal(rows[1, :9].reshape(3, 3), RGB[0, :, ::-1])
    assert (rows[:, 9:] == 0).all()


def test_to_bmp_row_padding_for_every_width():
    for w in range(1, 9):
        fb = np.ones((3, w, 4), np.float32)
        bmp = mm3e_cuda.to_bmp(fb)
        row = w * 3 + (4 - (w * 3) % 4) % 4
        assert row % 4 == 0 and len(bmp) == 54 + 3 * row
        assert int.from_bytes(bmp[34:38], "little") == 3 * row
