"""Writers for the V^3 PVM volume format and its DDS (differential data
stream) compression, written from the format description, for test fixtures:
the reader under test (csrc/host/readers.cpp) and the reference's own loader
(libs/file_utils/pvm.cpp, compiled by oracle/build_ref.py) must both decode
what these produce.

DDS bit stream (MSB first): skip-1 (2 bits), strip-1 (16 bits), then runs of
[count (7 bits, 0 ends the stream), code (3 bits; bits = code + 1 for
code >= 1, else 0), count residuals of 'bits' bits].  Value k is
(previous value [+ value[k-strip] - value[k-strip-1] once k > strip] +
residual - 2^bits/2) mod 256.  Before coding, the bytes are stored phase by
phase for an interleave of 'skip' (within blocks of skip * 2^24 bytes for
"DDS v3e").
"""
from __future__ import annotations

import numpy as np

BLOCK_V3E = 1 << 24


class _Bits:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value: int, bits: int):
        for i in range(bits - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                self.acc = 0
                self.n = 0

    def bytes(self) -> bytes:
        if self.n:
            return bytes(self.out) + bytes([self.acc << (8 - self.n)])
        return bytes(self.out)


def _phase_order(data: bytes, skip: int, block: int) -> bytes:
    if skip <= 1:
        return bytes(data)
    chunk = len(data) if block == 0 else skip * block
    out = bytearray()
    for base in range(0, len(data), chunk):
        part = data[base:base + chunk]
        for i in range(skip):
            out += part[i::skip]
    return bytes(out)


def _bits_for(d: int) -> int:
    # smallest representable width (0, 2..8) holding d in [-2^b/2, 2^b/2 - 1]
    if d == 0:
        return 0
    for b in range(2, 9):
        if -(1 << b) // 2 <= d <= (1 << b) // 2 - 1:
            return b
    return 8


def dds_encode(data: bytes, skip: int = 1, strip: int = 1, block: int = 0, run: int = 127) -> bytes:
    """The DDS stream (without the file magic) of data."""
    assert 1 <= skip <= 4 and 1 <= strip <= 65536 and 1 <= run <= 127
    s = np.frombuffer(_phase_order(data, skip, block), np.uint8).astype(np.int64)
    res = np.empty(len(s), np.int64)
    act = 0
    for k in range(len(s)):
        pred = act
        if strip > 1 and k > strip:
            pred += int(s[k - strip]) - int(s[k - strip - 1])
        res[k] = ((int(s[k]) - pred + 128) % 256) - 128
        act = int(s[k])
    w = _Bits()
    w.put(skip - 1, 2)
    w.put(strip - 1, 16)
    k = 0
    while k < len(res):
        n = min(run, len(res) - k)
        bits = max(_bits_for(int(d)) for d in res[k:k + n])
        w.put(n, 7)
        w.put(bits - 1 if bits > 1 else bits, 3)
        for d in res[k:k + n]:
            w.put(int(d) + (1 << bits) // 2, bits)
        k += n
    w.put(0, 7)
    return w.bytes()


def pvm_bytes(vol: np.ndarray, version: int = 3, scale=(1.0, 1.0, 1.0), comments=()) -> bytes:
    """A PVM file body for a (d, h, w) u8 or u16 volume (u16 stored low byte
    first, as the reference's loader assembles it)."""
    d, h, w = vol.shape
    comps = 1 if vol.dtype == np.uint8 else 2
    head = {1: "PVM\n", 2: "PVM2\n", 3: "PVM3\n"}[version]
    if version == 1:
        head += "".join(f"# {c}\n" for c in comments)
        head += f"{w} {h} {d}\n{comps}\n"
    else:
        head += f"{w} {h} {d}\n{scale[0]:g} {scale[1]:g} {scale[2]:g}\n{comps}\n"
    body = np.ascontiguousarray(vol).astype("<u2" if comps == 2 else np.uint8).tobytes()
    tail = b"\0\0\0\0" if version == 3 else b""  # empty description / courtesy / parameter / comment
    return head.encode() + body + tail


def dds_file(body: bytes, skip: int, strip: int, interleaved_blocks: bool = False) -> bytes:
    magic = b"DDS v3e\n" if interleaved_blocks else b"DDS v3d\n"
    return magic + dds_encode(body, skip, strip, BLOCK_V3E if interleaved_blocks else 0)
