"""Minimal multi-page TIFF writer: uncompressed grey pages, 8 or 16 bit,
either byte order, a chosen number of rows per strip (one page per z slice)."""
from __future__ import annotations

import struct

import numpy as np


def write_tiff(path, vol: np.ndarray, big_endian: bool = False, rows_per_strip: int | None = None) -> None:
    """vol [z][y][x] uint8 or uint16."""
    bo = ">" if big_endian else "<"
    if vol.ndim == 2:
        vol = vol[None]
    D, H, W = vol.shape
    bits = 8 if vol.dtype == np.uint8 else 16
    rps = rows_per_strip or H
    data = vol.astype(vol.dtype.newbyteorder(bo), copy=False)
    out = bytearray(b"MM\x00\x2a" if big_endian else b"II\x2a\x00")
    out += struct.pack(bo + "I", 0)  # first directory offset, patched below
    prev_next = 4

    def ent(tag, typ, count, value):
        if typ == 3 and count == 1:
            return struct.pack(bo + "HHI", tag, typ, count) + struct.pack(bo + "HH", value, 0)
        return struct.pack(bo + "HHII", tag, typ, count, value)

    for z in range(D):
        strips = []
        for r0 in range(0, H, rps):
            blob = data[z, r0:r0 + rps].tobytes()
            strips.append((len(out), len(blob)))
            out += blob
            if len(out) % 2:
                out += b"\x00"
        nst = len(strips)
        arr_off = len(out)
        for off, _ in strips:
            out += struct.pack(bo + "I", off)
        cnt_off = len(out)
        for _, n in strips:
            out += struct.pack(bo + "I", n)
        ifd = len(out)
        struct.pack_into(bo + "I", out, prev_next, ifd)
        entries = [ent(256, 4, 1, W), ent(257, 4, 1, H), ent(258, 3, 1, bits), ent(259, 3, 1, 1),
                   ent(262, 3, 1, 1), ent(273, 4, nst, arr_off if nst > 1 else strips[0][0]), ent(277, 3, 1, 1),
                   ent(278, 3, 1, rps), ent(279, 4, nst, cnt_off if nst > 1 else strips[0][1])]
        out += struct.pack(bo + "H", len(entries))
        for e in entries:
            out += e
        prev_next = len(out)
        out += struct.pack(bo + "I", 0)
    with open(path, "wb") as f:
        f.write(bytes(out))
