"""OpenEXR output of rendered images, in the form the reference writes them
(write_openexr_image, src/ref/reference_renderer.cpp:673-705, through
Image::write_exr, src/lib/image.cpp:163-225): a single-part scanline file,
channels B, G, R as HALF, no compression (one scanline per chunk) or ZIP
(16 scanlines per chunk), followed by YAR's custom attributes.

The layout follows the published OpenEXR file format: magic and version,
the header as (name, type, size, value) attributes ended by a null byte, the
chunk offset table, then the chunks (y, byte count, data).  ZIP chunks hold
the zlib stream of the scanline bytes after OpenEXR's byte split (even bytes,
then odd bytes) and delta predictor; a chunk that does not shrink is stored
raw."""
import struct
import zlib

import numpy as np

MAGIC = b"\x76\x2f\x31\x01"
NO_COMPRESSION, ZIP_COMPRESSION = 0, 3
HALF = 1
CHANNELS = (b"B", b"G", b"R")    # alphabetical, as the reference stores them


def to_half_bits(x):
    """float32 -> IEEE half bits, rounding to nearest with ties away from
    zero (the rounding of the reference's EXR writer; numpy's astype rounds
    ties to even), subnormal halves kept, overflow to infinity, NaN kept."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.int64)
    sign = (u >> 16) & 0x8000
    e = ((u >> 23) & 0xFF) - 127
    m = u & 0x7FFFFF
    out = np.zeros(u.shape, np.int64)
    nan_inf = e == 128
    out = np.where(nan_inf, 0x7C00 | np.where(m != 0, 0x200, 0), out)
    normal = (e >= -14) & (e <= 15)
    hn = ((e + 15) << 10) + ((m + 0x1000) >> 13)       # carry into the exponent rounds up across binades
    out = np.where(normal, np.minimum(hn, 0x7C00), out)
    out = np.where((e > 15) & ~nan_inf, 0x7C00, out)
    sub = (e < -14) & (e >= -25)
    shift = np.clip(-e - 1, 0, 63)                      # (m | 1 << 23) >> (shift) gives the subnormal mantissa
    full = m | (1 << 23)
    hs = (full + (np.int64(1) << (shift - 1).clip(0))) >> shift
    out = np.where(sub, hs, out)
    return (out | sign).astype(np.uint16)


def _attr(name, typ, value):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value


def yar_attributes(spp=0, variance=0.0, input_file="", device="gpu", build_asserts=1, build_version="0.0",
                   load_time=None, render_time=None):
    """YAR's custom attributes in the reference's order; the two timing
    attributes are written only when given (the reference's
    enable_varying_attributes)."""
    attrs = [("yar_build_version", "string", build_version.encode()),
             ("yar_build_asserts", "int", struct.pack("<i", int(build_asserts))),
             ("yar_render_device", "string", device.encode()),
             ("yar_input_file", "string", input_file.encode()),
             ("yar_spp", "int", struct.pack("<i", int(spp))),
             ("yar_variance", "float", struct.pack("<f", float(variance)))]
    if load_time is not None:
        attrs.append(("yar_load_time", "float", struct.pack("<f", float(load_time))))
    if render_time is not None:
        attrs.append(("yar_render_time", "float", struct.pack("<f", float(render_time))))
    return attrs


def _zip_encode(raw):
    b = np.frombuffer(raw, np.uint8)
    t = np.concatenate([b[0::2], b[1::2]]).astype(np.int16)
    d = t.copy()
    d[1:] = (t[1:] - t[:-1] + 128) & 0xFF
    return zlib.compress(d.astype(np.uint8).tobytes())


def _zip_decode(data, size):
    d = np.frombuffer(zlib.decompress(data), np.uint8).astype(np.int64)
    t = np.cumsum(np.concatenate([d[:1], d[1:] - 128])) & 0xFF
    t = t.astype(np.uint8)
    half = (size + 1) // 2
    out = np.empty(size, np.uint8)
    out[0::2] = t[:half]
    out[1::2] = t[half:]
    return out.tobytes()


def write_exr(path, rgb, compress=False, attributes=()):
    """rgb: (height, width, 3) float array, converted to HALF (to_half_bits)."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w, _ = rgb.shape
    chlist = b"".join(c + b"\0" + struct.pack("<iB3xii", HALF, 0, 1, 1) for c in CHANNELS) + b"\0"
    box = struct.pack("<iiii", 0, 0, w - 1, h - 1)
    header = (_attr("channels", "chlist", chlist) +
              _attr("compression", "compression", bytes([ZIP_COMPRESSION if compress else NO_COMPRESSION])) +
              _attr("dataWindow", "box2i", box) + _attr("displayWindow", "box2i", box) +
              _attr("lineOrder", "lineOrder", b"\0") + _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)) +
              _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)) +
              _attr("screenWindowWidth", "float", struct.pack("<f", float(w))) +
              b"".join(_attr(n, t, v) for n, t, v in attributes) + b"\0")
    half = to_half_bits(rgb).view(np.float16)
    # scanline bytes: per line, the B, G, R channel runs
    lines = np.stack([half[:, :, 2], half[:, :, 1], half[:, :, 0]], 1).reshape(h, -1)
    per = 16 if compress else 1
    chunks = []
    for y in range(0, h, per):
        raw = lines[y:y + per].tobytes()
        data = raw
        if compress:
            z = _zip_encode(raw)
            data = z if len(z) < len(raw) else raw
        chunks.append(struct.pack("<ii", y, len(data)) + data)
    pos = 8 + len(header) + 8 * len(chunks)
    offsets = []
    for c in chunks:
        offsets.append(pos)
        pos += len(c)
    with open(path, "wb") as f:
        f.write(MAGIC + struct.pack("<i", 2) + header + struct.pack("<%dQ" % len(chunks), *offsets) + b"".join(chunks))


def read_exr(path):
    """Reads the files write_exr (and the reference) writes: returns
    ((height, width, 3) float32 RGB, {attribute name: (type, bytes)})."""
    d = open(path, "rb").read()
    if d[:4] != MAGIC:
        raise ValueError("not an OpenEXR file")
    i = 8
    attrs = {}
    while d[i] != 0:
        j = d.index(b"\0", i)
        k = d.index(b"\0", j + 1)
        size = struct.unpack_from("<i", d, k + 1)[0]
        attrs[d[i:j].decode()] = (d[j + 1:k].decode(), d[k + 5:k + 5 + size])
        i = k + 5 + size
    i += 1
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    comp = attrs["compression"][1][0]
    per = {NO_COMPRESSION: 1, ZIP_COMPRESSION: 16}[comp]
    n = (h + per - 1) // per
    offsets = struct.unpack_from("<%dQ" % n, d, i)
    lines = np.empty((h, 3 * w), np.float16)
    for o in offsets:
        y, size = struct.unpack_from("<ii", d, o)
        rows = min(per, h - (y - y0))
        raw_size = rows * 3 * w * 2
        data = d[o + 8:o + 8 + size]
        if size < raw_size:
            data = _zip_decode(data, raw_size)
        lines[y - y0:y - y0 + rows] = np.frombuffer(data, np.float16).reshape(rows, 3 * w)
    bgr = lines.reshape(h, 3, w).astype(np.float32)
    return np.stack([bgr[:, 2], bgr[:, 1], bgr[:, 0]], 2), attrs
