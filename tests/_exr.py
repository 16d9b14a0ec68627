"""Minimal OpenEXR reader for the CLI's frames: single-part scanline files with
NO_COMPRESSION and FLOAT or HALF channels, parsed from the published file
layout (magic, version, attribute list, line offset table, chunks). Returns the
header attributes it understood and a dict of channel name -> (h, w) float32."""
from __future__ import annotations

import struct

import numpy as np


def _cstr(data: bytes, pos: int) -> tuple[str, int]:
    end = data.index(b"\0", pos)
    return data[pos:end].decode("ascii"), end + 1


def read_exr(path) -> tuple[dict, dict[str, np.ndarray]]:
    data = open(path, "rb").read()
    magic, version = struct.unpack_from("<ii", data, 0)
    if magic != 20000630:
        raise ValueError(f"{path}: not an OpenEXR file")
    if version & 0xFF != 2 or version & ~0xFF:
        raise ValueError(f"{path}: only single-part scanline files are read (version field {version:#x})")
    pos = 8
    attrs: dict = {}
    channels: list[tuple[str, int]] = []
    while data[pos] != 0:
        name, pos = _cstr(data, pos)
        kind, pos = _cstr(data, pos)
        (size,) = struct.unpack_from("<i", data, pos)
        pos += 4
        body = data[pos:pos + size]
        pos += size
        if kind == "chlist":
            q = 0
            while body[q] != 0:
                cname, q = _cstr(body, q)
                ptype, _plinear, xs, ys = struct.unpack_from("<iB3xii", body, q)
                q += 16
                if (xs, ys) != (1, 1):
                    raise ValueError("subsampled channels are not read")
                channels.append((cname, ptype))
            attrs[name] = [c for c, _ in channels]
        elif kind == "box2i":
            attrs[name] = struct.unpack("<4i", body)
        elif kind in ("compression", "lineOrder"):
            attrs[name] = body[0]
        elif kind == "float":
            attrs[name] = struct.unpack("<f", body)[0]
        elif kind == "v2f":
            attrs[name] = struct.unpack("<2f", body)
        else:
            attrs[name] = body
    pos += 1
    if attrs.get("compression") != 0:
        raise ValueError("only NO_COMPRESSION files are read")
    x0, y0, x1, y1 = attrs["dataWindow"]
    w, h = x1 - x0 + 1, y1 - y0 + 1
    offsets = struct.unpack_from(f"<{h}Q", data, pos)
    out = {c: np.zeros((h, w), np.float32) for c, _ in channels}
    for off in offsets:
        y, nbytes = struct.unpack_from("<ii", data, off)
        q = off + 8
        for cname, ptype in channels:
            if ptype == 2:
                row = np.frombuffer(data, "<f4", w, q)
                q += 4 * w
            elif ptype == 1:
                row = np.frombuffer(data, "<f2", w, q).astype(np.float32)
                q += 2 * w
            else:
                raise ValueError("UINT channels are not read")
            out[cname][y - y0] = row
        if q != off + 8 + nbytes:
            raise ValueError("chunk size does not match its channels")
    return attrs, out
