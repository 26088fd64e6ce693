"""Volume and image files for visual diffing (host side, numpy + zlib only).

* PNG: RGBA images from the renderer (float RGBA in [0, 1], row 0 = top)
  written as 8-bit RGBA (filter type 0 rows, one IDAT chunk), and read back.
* .vol: one pyramid level as stored on the device (RGBA32F or the packed
  BF16/FP16 word), after a 32-byte header: magic b"CGVOL\\x01", format (u8),
  reserved (u16), level (u32), dimension (u32 x 3), bytes per voxel (u32),
  then dimension^3 voxels, x fastest.
"""
import struct
import zlib

import numpy as np

_PNG_SIG = b"\x89PNG\r\n\x1a\n"
_VOL_MAGIC = b"CGVOL\x01"


def _chunk(kind, data):
    body = kind + data
    return struct.pack(">I", len(data)) + body + struct.pack(">I", zlib.crc32(body) & 0xFFFFFFFF)


def to_rgba8(image):
    """Float RGBA (H, W, 4) -> uint8, clamped to [0, 1] and rounded."""
    img = np.asarray(image, np.float64)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("expected an (H, W, 4) RGBA image")
    return np.clip(np.rint(np.clip(img, 0.0, 1.0) * 255.0), 0, 255).astype(np.uint8)


def save_png(path, image):
    """Write a float RGBA image (or an (H, W, 4) uint8 array) as an 8-bit RGBA PNG."""
    a = np.asarray(image)
    rgba = a if a.dtype == np.uint8 else to_rgba8(a)
    h, w = rgba.shape[:2]
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))
    ihdr = struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)
    with open(path, "wb") as f:
        f.write(_PNG_SIG + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(raw, 6)) +
                _chunk(b"IEND", b""))


def load_png(path):
    """Read an 8-bit RGBA PNG written by save_png -> (H, W, 4) uint8."""
    with open(path, "rb") as f:
        data = f.read()
    if not data.startswith(_PNG_SIG):
        raise ValueError(f"{path}: not a PNG file")
    pos, ihdr, idat = 8, None, b""
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if zlib.crc32(kind + body) & 0xFFFFFFFF != struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]:
            raise ValueError(f"{path}: bad CRC in {kind!r}")
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    if ihdr is None or ihdr[2:5] != (8, 6, 0):
        raise ValueError(f"{path}: only 8-bit RGBA PNGs are supported")
    w, h = ihdr[0], ihdr[1]
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    if np.any(raw[:, 0] != 0):
        raise ValueError(f"{path}: only filter type 0 rows are supported")
    return raw[:, 1:].reshape(h, w, 4).copy()


def save_volume(path, volume, level=0):
    """Write one level of a CloudVolume (as stored) to a .vol file."""
    data = np.ascontiguousarray(volume.read_level(level))
    info = volume.info()
    n = int(info.level_dim[level])
    bpv = int(info.bytes_per_voxel)
    header = _VOL_MAGIC + struct.pack("<BHIIIII", int(info.format), 0, int(level), n, n, n, bpv)
    header += b"\x00" * (32 - len(header))
    with open(path, "wb") as f:
        f.write(header)
        f.write(data.tobytes())


def load_volume(path):
    """Read a .vol file -> (array, meta).  RGBA32F levels come back as
    (n, n, n, 4) float32, packed BF16/FP16 levels as (n, n, n) uint32."""
    with open(path, "rb") as f:
        head = f.read(32)
        if not head.startswith(_VOL_MAGIC):
            raise ValueError(f"{path}: not a .vol file")
        fmt, _, level, nx, ny, nz, bpv = struct.unpack("<BHIIIII", head[6:29])
        body = f.read()
    count = nx * ny * nz
    if len(body) != count * bpv:
        raise ValueError(f"{path}: {len(body)} data bytes, expected {count * bpv}")
    if bpv == 16:
        arr = np.frombuffer(body, np.float32).reshape(nz, ny, nx, 4)
    elif bpv == 4:
        arr = np.frombuffer(body, np.uint32).reshape(nz, ny, nx)
    else:
        raise ValueError(f"{path}: unsupported voxel size {bpv}")
    return arr.copy(), dict(format=fmt, level=level, dims=(nx, ny, nz), bytes_per_voxel=bpv)


def unpack_bf16_fp16(words):
    """Packed BF16 (R, low half) / FP16 (G, high half) words -> (R, G) float32."""
    w = np.asarray(words, np.uint32)
    r = (w << np.uint32(16)).view(np.float32)
    g = (w >> np.uint32(16)).astype(np.uint16).view(np.float16).astype(np.float32)
    return r, g
