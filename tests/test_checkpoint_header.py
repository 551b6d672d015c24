"""Checkpoint images on the host: the header a checkpoint starts with, read
and checked by poe_checkpoint_info without a GPU.

An image is the header (poe_checkpoint_header) followed by its payload; the
reader accepts a version-2 header whose payload is present and matches its
checksum, and rejects anything else with a status code.  The images here are
built byte by byte in Python; the checksum is restated from its definition
(64-bit words: h = (h ^ w) * 0x100000001b3, h ^= h >> 29, then the tail
bytes h = (h ^ b) * 0x100000001b3, from h = 0x9e3779b97f4a7c15).
"""
import ctypes as C

import numpy as np
import pytest

M64 = (1 << 64) - 1


def checksum(payload: bytes) -> int:
    h = 0x9e3779b97f4a7c15
    n8 = len(payload) // 8 * 8
    for w in np.frombuffer(payload[:n8], "<u8").tolist():
        h = ((h ^ w) * 0x100000001b3) & M64
        h ^= h >> 29
    for b in payload[n8:]:
        h = ((h ^ b) * 0x100000001b3) & M64
    return h


def image(payload=b"", version=2, magic=b"POE2DCK1", **fields):
    from poe2d_gb300 import _lib as L
    h = L.CheckpointHeader()
    h.magic = magic
    h.version = version
    h.header_bytes = C.sizeof(h)
    h.NX, h.NZ, h.steps, h.nrec, h.dt = 40, 30, 17, 3, 5e-5
    for k, v in fields.items():
        setattr(h, k, v)
    h.payload_bytes = len(payload)
    h.checksum = checksum(payload)
    return bytes(h) + payload


def test_header_is_read_back():
    import poe2d_gb300 as P
    payload = np.arange(1003, dtype=np.uint8).tobytes()      # tail bytes past the last 8-byte word
    info = P.checkpoint_info(image(payload, prof_hash=0x1234, coef_hash=0xabcdef, rec_hash=7, dx=0.5))
    assert info["magic"] == b"POE2DCK1" and info["version"] == 2
    assert (info["NX"], info["NZ"], info["steps"], info["nrec"]) == (40, 30, 17, 3)
    assert (info["prof_hash"], info["coef_hash"], info["rec_hash"]) == (0x1234, 0xabcdef, 7)
    assert info["dx"] == 0.5 and info["dt"] == np.float32(5e-5)
    assert info["payload_bytes"] == 1003


def test_header_rejects_other_versions_and_short_or_corrupt_images():
    import poe2d_gb300 as P
    payload = bytes(range(256)) * 4
    good = image(payload)
    P.checkpoint_info(good)
    with pytest.raises(P.PoeError) as e:
        P.checkpoint_info(image(payload, version=1))           # images without the model hashes
    assert e.value.status == 1
    with pytest.raises(P.PoeError) as e:
        P.checkpoint_info(image(payload, magic=b"NOTACKPT"))
    assert e.value.status == 1
    with pytest.raises(P.PoeError) as e:
        P.checkpoint_info(good[:-1])                           # payload cut short
    assert e.value.status == 1
    with pytest.raises(P.PoeError) as e:
        P.checkpoint_info(good[:40])                           # not even a header
    assert e.value.status == 1
    bad = bytearray(good)
    bad[-100] ^= 0x10
    with pytest.raises(P.PoeError) as e:
        P.checkpoint_info(bytes(bad))
    assert e.value.status == 7                                 # POE_EIO: checksum
