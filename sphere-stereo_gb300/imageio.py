"""Panorama files: 8-bit PNG and float32 OpenEXR writers and readers, host-side, off the timed
path (the reference writes them with cv2.imwrite, python/utils.py:253-260, and reads ground truth
with cv2.imread, python/utils.py:215-218; cv2 is not a dependency here).

Channel order follows cv2: a [rows, cols, 3] array holds B, G, R (the order the reference's
images keep from cv2.imread), so the PNG file's R channel is the array's last channel.  A
[rows, cols] float32 array is written as an EXR with the single channel "Y" (cv2's layout for
one-channel images); three-channel float arrays as B, G, R channels.

Formats (public specifications):
  - PNG (ISO/IEC 15948): signature, IHDR, one zlib-compressed IDAT, IEND; 8-bit greyscale or
    RGB, filter type 0 on write, all five filter types on read, no interlace.
  - OpenEXR 2 scanline files: magic 20000630, version 2, header attributes, offset table,
    chunks of scanlines; FLOAT (32-bit) or HALF pixels; NO_COMPRESSION (1 line per chunk) on
    write, NO / ZIPS (1 line) / ZIP (16 lines) compression on read (zlib data, then the
    format's byte-interleave and delta predictor undone).
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np

_PNG_SIGNATURE = b"\x89PNG\r\n\x1a\n"
_EXR_MAGIC = 20000630


# --------------------------------------------------------------------------------------------
# PNG
# --------------------------------------------------------------------------------------------
def _png_chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def encode_png(image: np.ndarray, level: int = 6) -> bytes:
    """PNG bytes of a uint8 [rows, cols] (greyscale) or [rows, cols, 3] (B, G, R) array."""
    a = np.asarray(image)
    if a.dtype != np.uint8:
        raise TypeError(f"PNG images must be uint8 (got {a.dtype})")
    if a.ndim == 2:
        colour_type, rows_data = 0, a
    elif a.ndim == 3 and a.shape[2] == 3:
        colour_type, rows_data = 2, a[:, :, ::-1]  # B, G, R -> the file's R, G, B
    else:
        raise ValueError(f"PNG images must be [rows, cols] or [rows, cols, 3] (got {a.shape})")
    rows, cols = a.shape[:2]
    raw = np.ascontiguousarray(rows_data).reshape(rows, -1)
    scan = np.empty((rows, raw.shape[1] + 1), np.uint8)
    scan[:, 0] = 0  # filter type None
    scan[:, 1:] = raw
    ihdr = struct.pack(">IIBBBBB", cols, rows, 8, colour_type, 0, 0, 0)
    return (_PNG_SIGNATURE + _png_chunk(b"IHDR", ihdr) + _png_chunk(b"IDAT", zlib.compress(scan.tobytes(), level))
            + _png_chunk(b"IEND", b""))


def _paeth(a: np.ndarray, b: np.ndarray, c: np.ndarray) -> np.ndarray:
    a16, b16, c16 = a.astype(np.int16), b.astype(np.int16), c.astype(np.int16)
    p = a16 + b16 - c16
    pa, pb, pc = np.abs(p - a16), np.abs(p - b16), np.abs(p - c16)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c)).astype(np.uint8)


def decode_png(data: bytes) -> np.ndarray:
    """uint8 array of an 8-bit greyscale, RGB or RGBA PNG ([rows, cols] or [rows, cols, 3|4], colour
    channels as B, G, R like cv2.imread with IMREAD_UNCHANGED)."""
    if data[:8] != _PNG_SIGNATURE:
        raise ValueError("not a PNG file")
    pos, idat, header = 8, [], None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        (crc,) = struct.unpack(">I", data[pos + 8 + length:pos + 12 + length])
        if zlib.crc32(kind + body) & 0xFFFFFFFF != crc:
            raise ValueError(f"PNG chunk {kind!r}: CRC mismatch")
        if kind == b"IHDR":
            header = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + length
    if header is None:
        raise ValueError("PNG without IHDR")
    cols, rows, depth, colour_type, _, _, interlace = header
    channels = {0: 1, 2: 3, 6: 4}.get(colour_type)
    if depth != 8 or channels is None or interlace != 0:
        raise ValueError(f"unsupported PNG: depth {depth}, colour type {colour_type}, interlace {interlace}")
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8)
    stride = cols * channels
    raw = raw[:rows * (stride + 1)].reshape(rows, stride + 1)
    out = np.zeros((rows, stride), np.uint8)
    prev = np.zeros(stride, np.uint8)
    for y in range(rows):
        f, line = raw[y, 0], raw[y, 1:].copy()
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev).astype(np.uint8)
        else:  # 1 (sub), 3 (average), 4 (Paeth) depend on the reconstructed left neighbour
            cur = np.zeros(stride, np.uint8)
            for x in range(stride):
                left = cur[x - channels] if x >= channels else 0
                upleft = prev[x - channels] if x >= channels else 0
                if f == 1:
                    pred = left
                elif f == 3:
                    pred = (int(left) + int(prev[x])) // 2
                elif f == 4:
                    pred = _paeth(np.uint8(left), prev[x], np.uint8(upleft))
                else:
                    raise ValueError(f"PNG filter type {f}")
                cur[x] = (int(line[x]) + int(pred)) & 0xFF
        out[y] = cur
        prev = cur
    img = out.reshape(rows, cols, channels)
    if channels == 1:
        return img[:, :, 0]
    if channels == 3:
        return img[:, :, ::-1].copy()
    return img[:, :, [2, 1, 0, 3]].copy()


# --------------------------------------------------------------------------------------------
# OpenEXR
# --------------------------------------------------------------------------------------------
_PIXEL_HALF, _PIXEL_FLOAT = 1, 2
_NO_COMPRESSION, _ZIPS, _ZIP = 0, 2, 3


def _attr(name: str, kind: str, value: bytes) -> bytes:
    return name.encode() + b"\0" + kind.encode() + b"\0" + struct.pack("<i", len(value)) + value


def encode_exr(image: np.ndarray) -> bytes:
    """Uncompressed scanline OpenEXR bytes of a float32 [rows, cols] (channel Y) or
    [rows, cols, 3] (B, G, R) array, FLOAT pixels."""
    a = np.asarray(image)
    if a.dtype != np.float32:
        raise TypeError(f"EXR images must be float32 (got {a.dtype})")
    if a.ndim == 2:
        names, planes = ["Y"], [a]
    elif a.ndim == 3 and a.shape[2] == 3:
        names, planes = ["B", "G", "R"], [a[:, :, 0], a[:, :, 1], a[:, :, 2]]
    else:
        raise ValueError(f"EXR images must be [rows, cols] or [rows, cols, 3] (got {a.shape})")
    rows, cols = a.shape[:2]
    order = sorted(range(len(names)), key=lambda i: names[i])  # channels are stored by name
    chlist = b"".join(names[i].encode() + b"\0" + struct.pack("<iBBBBii", _PIXEL_FLOAT, 0, 0, 0, 0, 1, 1)
                      for i in order) + b"\0"
    box = struct.pack("<iiii", 0, 0, cols - 1, rows - 1)
    header = (struct.pack("<ii", _EXR_MAGIC, 2)
              + _attr("channels", "chlist", chlist)
              + _attr("compression", "compression", bytes([_NO_COMPRESSION]))
              + _attr("dataWindow", "box2i", box)
              + _attr("displayWindow", "box2i", box)
              + _attr("lineOrder", "lineOrder", bytes([0]))
              + _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
              + _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
              + _attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
              + b"\0")
    line_bytes = 4 * cols * len(names)
    table_start = len(header)
    first = table_start + 8 * rows
    offsets = struct.pack(f"<{rows}Q", *[first + y * (8 + line_bytes) for y in range(rows)])
    stacked = np.stack([np.ascontiguousarray(planes[i], dtype="<f4") for i in order], axis=1)  # [rows, ch, cols]
    chunks = bytearray()
    for y in range(rows):
        chunks += struct.pack("<ii", y, line_bytes) + stacked[y].tobytes()
    return header + offsets + bytes(chunks)


def _read_attributes(data: bytes, pos: int) -> tuple[dict, int]:
    attrs = {}
    while data[pos] != 0:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        end2 = data.index(b"\0", end + 1)
        kind = data[end + 1:end2].decode()
        (size,) = struct.unpack("<i", data[end2 + 1:end2 + 5])
        attrs[name] = (kind, data[end2 + 5:end2 + 5 + size])
        pos = end2 + 5 + size
    return attrs, pos + 1


def _unzip_exr(block: bytes, expected: int) -> bytes:
    raw = np.frombuffer(zlib.decompress(block), np.uint8)
    if raw.size != expected:
        raise ValueError("EXR ZIP block of unexpected size")
    t = raw.astype(np.int32)
    t = np.cumsum(np.concatenate([t[:1], t[1:] - 128])) & 0xFF  # undo the delta predictor
    t = t.astype(np.uint8)
    half = (t.size + 1) // 2
    out = np.empty_like(t)
    out[0::2] = t[:half]  # undo the byte interleave
    out[1::2] = t[half:]
    return out.tobytes()


def decode_exr(data: bytes) -> np.ndarray:
    """float32 array of a scanline OpenEXR file (NO, ZIPS or ZIP compression): [rows, cols] for
    one channel, else [rows, cols, channels] with B, G, R (then the rest by name) first."""
    (magic, version) = struct.unpack("<ii", data[:8])
    if magic != _EXR_MAGIC:
        raise ValueError("not an OpenEXR file")
    if version & 0x200:
        raise ValueError("tiled OpenEXR files are not supported")
    attrs, pos = _read_attributes(data, 8)
    comp = attrs["compression"][1][0]
    lines_per_chunk = {_NO_COMPRESSION: 1, _ZIPS: 1, _ZIP: 16}.get(comp)
    if lines_per_chunk is None:
        raise ValueError(f"unsupported EXR compression {comp}")
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    cols, rows = x1 - x0 + 1, y1 - y0 + 1
    chl = attrs["channels"][1]
    channels, p = [], 0
    while chl[p] != 0:
        end = chl.index(b"\0", p)
        name = chl[p:end].decode()
        ptype, _, _, _, _, xs, ys = struct.unpack("<iBBBBii", chl[end + 1:end + 17])
        if (xs, ys) != (1, 1) or ptype not in (_PIXEL_HALF, _PIXEL_FLOAT):
            raise ValueError(f"unsupported EXR channel {name}")
        channels.append((name, ptype))
        p = end + 17
    chunk_count = -(-rows // lines_per_chunk)
    offsets = struct.unpack(f"<{chunk_count}Q", data[pos:pos + 8 * chunk_count])
    sizes = [2 if t == _PIXEL_HALF else 4 for _, t in channels]
    planes = {name: np.empty((rows, cols), np.float32) for name, _ in channels}
    for off in offsets:
        (yc, size) = struct.unpack("<ii", data[off:off + 8])
        n = min(lines_per_chunk, y1 - yc + 1)
        expected = n * cols * sum(sizes)
        block = data[off + 8:off + 8 + size]
        if comp != _NO_COMPRESSION and size < expected:
            block = _unzip_exr(block, expected)
        q = 0
        for line in range(n):
            for (name, ptype), sz in zip(channels, sizes):
                dt = "<f2" if ptype == _PIXEL_HALF else "<f4"
                planes[name][yc - y0 + line] = np.frombuffer(block, dt, cols, q).astype(np.float32)
                q += sz * cols
    names = [n for n, _ in channels]
    if len(names) == 1:
        return planes[names[0]]
    ordered = [n for n in ("B", "G", "R") if n in planes] + sorted(n for n in names if n not in ("B", "G", "R"))
    return np.stack([planes[n] for n in ordered], axis=2)


# --------------------------------------------------------------------------------------------
# Files
# --------------------------------------------------------------------------------------------
def imwrite(path: str, image: np.ndarray) -> bool:
    """Writes a .png (uint8) or .exr (float32) file; returns True as cv2.imwrite does."""
    ext = os.path.splitext(path)[1].lower()
    if ext == ".png":
        data = encode_png(image)
    elif ext == ".exr":
        data = encode_exr(image)
    else:
        raise ValueError(f"unsupported image file type {ext!r} (.png or .exr)")
    with open(path, "wb") as f:
        f.write(data)
    return True


def imread(path: str) -> np.ndarray | None:
    """Reads a .png or .exr file as cv2.imread(path, IMREAD_UNCHANGED) would; None when the file
    is missing or unreadable (cv2's behaviour)."""
    try:
        with open(path, "rb") as f:
            data = f.read()
    except OSError:
        return None
    try:
        if data[:8] == _PNG_SIGNATURE:
            return decode_png(data)
        if data[:4] == struct.pack("<i", _EXR_MAGIC):
            return decode_exr(data)
    except (ValueError, KeyError, zlib.error, struct.error):
        return None
    return None


def save_rgbd_panorama(rgbd_panoramas: dict, filename: str, dataset_path: str) -> None:
    """python/utils.py:252-260: writes output/rgb_<name>.png and output/inv_distance_<name>.exr
    under dataset_path for rgbd_panoramas[filename] ({"rgb": uint8 [rows, cols, 3],
    "inv_distance": float32 [rows, cols]}, numpy arrays or CPU/CUDA tensors); a missing key is
    ignored, as in the reference."""
    try:
        pano = rgbd_panoramas[filename]
    except KeyError:
        return
    save_name = os.path.splitext(filename)[0]
    imwrite(os.path.join(dataset_path, "output/rgb_" + save_name + ".png"), _numpy(pano["rgb"]))
    imwrite(os.path.join(dataset_path, "output/inv_distance_" + save_name + ".exr"), _numpy(pano["inv_distance"]))


def _numpy(a) -> np.ndarray:
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a)
