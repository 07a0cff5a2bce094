"""Surrogate training-data files: a stream of samples (one scene at one time step) written while
the batched solver runs, read back for training. No counterpart in the reference.

File layout (little-endian):
    file header   b"WCDATA01", uint32 version (1), uint32 record header bytes
    record        header: b"WCSMPL01", uint32 scene, uint32 step, uint64 n, float32 dt,
                  uint32 reserved, wc_params (the scene's parameters), uint64 checksum of the
                  record's arrays (BLAKE2b, 8-byte digest)
                  arrays: particles[n] (wc_particle, 32 bytes, id order), history[5][n][4]
                  float32, target[n][4] float32 (the SPH acceleration, w = 0)
Records are appended as they are produced, so a long run needs no memory beyond one frame.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import struct
from pathlib import Path

import numpy as np

from . import _abi as A
from .surrogate import HISTORY, Sample

FILE_MAGIC = b"WCDATA01"
RECORD_MAGIC = b"WCSMPL01"
VERSION = 1
_REC = struct.Struct("<8sIIQfI")  # magic, scene, step, n, dt, reserved
_PARAMS_BYTES = C.sizeof(A.Params)
RECORD_HEADER_BYTES = _REC.size + _PARAMS_BYTES + 8


def _checksum(arrays) -> int:
    """BLAKE2b digest (8 bytes) of the arrays' bytes, in order."""
    h = hashlib.blake2b(digest_size=8)
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return int.from_bytes(h.digest(), "little")


class DatasetWriter:
    """Append samples to a dataset file."""

    def __init__(self, path, params: list):
        self.path = Path(path)
        self.params = params
        self.fh = open(self.path, "wb")
        self.fh.write(FILE_MAGIC + struct.pack("<II", VERSION, RECORD_HEADER_BYTES))
        self.count = 0

    def write(self, smp: Sample) -> None:
        n = smp.state.shape[0]
        state = np.ascontiguousarray(smp.state, dtype=A.PARTICLE_DTYPE)
        hist = np.ascontiguousarray(smp.hist, dtype=np.float32)
        target = np.ascontiguousarray(smp.target, dtype=np.float32)
        if hist.shape != (HISTORY, n, 4) or target.shape != (n, 4):
            raise A.WatercubeError(A.WC_ERR_INVALID_ARG, "sample arrays have inconsistent shapes")
        p = self.params[smp.scene]
        self.fh.write(_REC.pack(RECORD_MAGIC, smp.scene, smp.step, n, float(smp.dt), 0))
        self.fh.write(bytes(p))
        self.fh.write(struct.pack("<Q", _checksum([state, hist, target])))
        for a in (state, hist, target):
            self.fh.write(a.tobytes())
        self.count += 1

    def close(self) -> None:
        if self.fh is not None:
            self.fh.close()
            self.fh = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_dataset(path, verify: bool = True):
    """Yield (params, Sample) for every record of a dataset file."""
    with open(path, "rb") as fh:
        head = fh.read(16)
        if len(head) != 16 or head[:8] != FILE_MAGIC:
            raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"{path} is not a dataset file")
        version, rec_bytes = struct.unpack("<II", head[8:])
        if version != VERSION or rec_bytes != RECORD_HEADER_BYTES:
            raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"{path}: version {version}, record header {rec_bytes} bytes")
        while True:
            raw = fh.read(RECORD_HEADER_BYTES)
            if not raw:
                return
            if len(raw) != RECORD_HEADER_BYTES:
                raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"{path}: truncated record header")
            magic, scene, step, n, dt, _ = _REC.unpack(raw[:_REC.size])
            if magic != RECORD_MAGIC:
                raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"{path}: bad record magic")
            params = A.Params.from_buffer_copy(raw[_REC.size:_REC.size + _PARAMS_BYTES])
            (checksum,) = struct.unpack("<Q", raw[_REC.size + _PARAMS_BYTES:])
            sizes = (n * A.PARTICLE_DTYPE.itemsize, HISTORY * n * 16, n * 16)
            bufs = [fh.read(s) for s in sizes]
            if any(len(b) != s for b, s in zip(bufs, sizes)):
                raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"{path}: truncated record")
            state = np.frombuffer(bufs[0], dtype=A.PARTICLE_DTYPE).copy()
            hist = np.frombuffer(bufs[1], dtype=np.float32).reshape(HISTORY, n, 4).copy()
            target = np.frombuffer(bufs[2], dtype=np.float32).reshape(n, 4).copy()
            if verify and _checksum([state, hist, target]) != checksum:
                raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"{path}: record {scene}/{step} fails its checksum")
            yield params, Sample(scene, step, float(dt), state, hist, target)
