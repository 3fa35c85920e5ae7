"""A small self-checking container for named numpy arrays (network weights,
standardizers, calibration tables): a fixed header, a JSON index and the raw
array bytes, followed by a SHA-256 of everything before it.

    b"SCTLCKPT" | u32 version | u64 index length | index (UTF-8 JSON) | payload | sha256

The index lists every array's name, dtype, shape and byte offset in the
payload, and a free-form "meta" object.  Loading verifies the magic, the
version and the checksum before it trusts a byte.
"""
from __future__ import annotations

import hashlib
import json
import struct

import numpy as np

MAGIC = b"SCTLCKPT"
VERSION = 1


class CheckpointError(ValueError):
    pass


def dumps(arrays: dict, meta: dict | None = None) -> bytes:
    """Serialise {name: array} (and a JSON-able meta dict)."""
    index, chunks, off = [], [], 0
    for name, a in arrays.items():
        a = np.asarray(a)
        if a.dtype.kind not in "fiub":
            raise CheckpointError(f"array {name!r}: unsupported dtype {a.dtype}")
        raw = a.tobytes(order="C")
        index.append({"name": str(name), "dtype": a.dtype.str, "shape": list(a.shape), "offset": off,
                      "nbytes": len(raw)})
        chunks.append(raw)
        off += len(raw)
    head = json.dumps({"arrays": index, "meta": meta or {}}, sort_keys=True).encode()
    body = MAGIC + struct.pack("<IQ", VERSION, len(head)) + head + b"".join(chunks)
    return body + hashlib.sha256(body).digest()


def loads(blob: bytes):
    """Inverse of dumps: returns ({name: array}, meta); raises CheckpointError on any damage."""
    if len(blob) < len(MAGIC) + 12 + 32 or blob[:len(MAGIC)] != MAGIC:
        raise CheckpointError("not a checkpoint (bad magic or too short)")
    body, digest = blob[:-32], blob[-32:]
    if hashlib.sha256(body).digest() != digest:
        raise CheckpointError("checksum mismatch")
    version, hlen = struct.unpack("<IQ", body[len(MAGIC):len(MAGIC) + 12])
    if version != VERSION:
        raise CheckpointError(f"unsupported version {version}")
    p0 = len(MAGIC) + 12
    head = json.loads(body[p0:p0 + hlen].decode())
    payload = memoryview(body)[p0 + hlen:]
    arrays = {}
    for e in head["arrays"]:
        o, n = e["offset"], e["nbytes"]
        if o < 0 or o + n > len(payload):
            raise CheckpointError(f"array {e['name']!r} out of bounds")
        a = np.frombuffer(payload[o:o + n], dtype=np.dtype(e["dtype"])).reshape(e["shape"]).copy()
        arrays[e["name"]] = a
    return arrays, head.get("meta", {})


def save(path: str, arrays: dict, meta: dict | None = None) -> None:
    with open(path, "wb") as fh:
        fh.write(dumps(arrays, meta))


def load(path: str):
    with open(path, "rb") as fh:
        return loads(fh.read())
