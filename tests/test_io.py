"""Volume (.vol) and image (PNG) files: round trips on the host, and one
GPU case that dumps a voxelized level and an image and reads them back."""
import struct
import zlib

import numpy as np
import pytest

from cloudgb import io as cio


def test_png_round_trip_float_and_uint8(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.uniform(-0.2, 1.2, (37, 53, 4)).astype(np.float32)
    p = tmp_path / "a.png"
    cio.save_png(p, img)
    back = cio.load_png(p)
    assert back.shape == (37, 53, 4) and back.dtype == np.uint8
    assert np.array_equal(back, cio.to_rgba8(img))
    u8 = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    cio.save_png(tmp_path / "b.png", u8)
    assert np.array_equal(cio.load_png(tmp_path / "b.png"), u8)


def test_png_quantization_and_layout(tmp_path):
    img = np.zeros((2, 3, 4), np.float32)
    img[0, 0] = (1.0, 0.5, 0.0, 1.0)      # 0.5 * 255 = 127.5 -> 128 (round half even)
    img[1, 2] = (0.25, 2.0, -1.0, 0.0)
    cio.save_png(tmp_path / "q.png", img)
    data = (tmp_path / "q.png").read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", data[16:24])
    assert (w, h) == (3, 2)
    back = cio.load_png(tmp_path / "q.png")
    assert tuple(back[0, 0]) == (255, 128, 0, 255)
    assert tuple(back[1, 2]) == (64, 255, 0, 0)


def test_png_rejects_corruption(tmp_path):
    p = tmp_path / "c.png"
    cio.save_png(p, np.ones((4, 4, 4), np.float32))
    data = bytearray(p.read_bytes())
    data[40] ^= 0xFF                       # inside IDAT
    p.write_bytes(bytes(data))
    with pytest.raises(ValueError, match="CRC"):
        cio.load_png(p)
    (tmp_path / "x.png").write_bytes(b"not a png")
    with pytest.raises(ValueError):
        cio.load_png(tmp_path / "x.png")
    with pytest.raises(ValueError):
        cio.save_png(tmp_path / "y.png", np.zeros((4, 4, 3), np.float32))


class _FakeVolume:
    """Stands in for CloudVolume: read_level + info as the library returns them."""

    def __init__(self, levels, fmt, bpv):
        self.levels, self.fmt, self.bpv = levels, fmt, bpv

    def read_level(self, level):
        return self.levels[level]

    def info(self):
        class Info:
            pass
        inf = Info()
        inf.format = self.fmt
        inf.bytes_per_voxel = self.bpv
        inf.level_dim = [lv.shape[0] for lv in self.levels]
        return inf


def test_vol_round_trip_rgba32f_and_packed(tmp_path):
    rng = np.random.default_rng(1)
    f32 = [rng.random((8 >> l, 8 >> l, 8 >> l, 4), dtype=np.float32) for l in range(3)]
    vol = _FakeVolume(f32, 0, 16)
    for l in range(3):
        cio.save_volume(tmp_path / f"f{l}.vol", vol, l)
        arr, meta = cio.load_volume(tmp_path / f"f{l}.vol")
        assert np.array_equal(arr, f32[l])
        assert meta == dict(format=0, level=l, dims=(8 >> l,) * 3, bytes_per_voxel=16)
    packed = [rng.integers(0, 2 ** 32, (6, 6, 6), dtype=np.uint32)]
    cio.save_volume(tmp_path / "p.vol", _FakeVolume(packed, 1, 4), 0)
    arr, meta = cio.load_volume(tmp_path / "p.vol")
    assert arr.dtype == np.uint32 and np.array_equal(arr, packed[0])
    assert meta["format"] == 1 and meta["bytes_per_voxel"] == 4
    assert (tmp_path / "p.vol").stat().st_size == 32 + 4 * 216


def test_vol_rejects_truncation(tmp_path):
    vol = _FakeVolume([np.zeros((4, 4, 4, 4), np.float32)], 0, 16)
    cio.save_volume(tmp_path / "t.vol", vol)
    data = (tmp_path / "t.vol").read_bytes()
    (tmp_path / "t.vol").write_bytes(data[:-16])
    with pytest.raises(ValueError, match="expected"):
        cio.load_volume(tmp_path / "t.vol")
    (tmp_path / "bad.vol").write_bytes(b"\x00" * 64)
    with pytest.raises(ValueError, match="not a .vol"):
        cio.load_volume(tmp_path / "bad.vol")


def test_unpack_bf16_fp16():
    r = np.array([1.0, -2.5, 0.15625], np.float32)
    g = np.array([0.5, 3.0, -0.25], np.float16)
    words = (r.view(np.uint32) >> 16) | (g.view(np.uint16).astype(np.uint32) << 16)
    ur, ug = cio.unpack_bf16_fp16(words)
    assert np.array_equal(ur, r) and np.array_equal(ug, g.astype(np.float32))


@pytest.mark.gpu
def test_gpu_volume_and_image_dump(ctx, tmp_path):
    import cloudgb
    from cloudgb import configs, workload
    cfg = configs.SMALL_64
    wl = workload.build(cfg)
    for fmt in (cloudgb.FORMAT_RGBA32F, cloudgb.FORMAT_BF16_FP16):
        vol = cloudgb.CloudVolume(cfg["dim"], configs.VOLUME_BOUNDS, configs.VOLUME_POSITION,
                                  cfg["mips"], fmt=fmt, ctx=ctx)
        vol.set_billboards(wl.positions, wl.scales, wl.densities)
        vol.update()
        sun = cloudgb.Sun(wl.sun_direction, *wl.sun_map)
        cloudgb.VoxelizeShader().voxelize(vol, sun)
        for l in range(cfg["mips"]):
            p = tmp_path / f"v{fmt}_{l}.vol"
            cio.save_volume(p, vol, l)
            arr, meta = cio.load_volume(p)
            assert np.array_equal(arr, vol.read_level(l))
            assert meta["format"] == fmt and meta["level"] == l
        shader = cloudgb.ConeTraceShader(**wl.shader_kwargs())
        img = shader.coneTrace(vol, workload.make_camera(wl.cameras[0]))
        cio.save_png(tmp_path / f"img{fmt}.png", img)
        assert np.array_equal(cio.load_png(tmp_path / f"img{fmt}.png"), cio.to_rgba8(img))
        vol.close()
