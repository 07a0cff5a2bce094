"""Snapshot files (C reader, no GPU: files written here in the documented layout) and the
surrogate dataset files (write / read round trip, corruption detection)."""
import ctypes as C
import struct

import numpy as np
import pytest

from watercube_gb300 import _abi
from watercube_gb300.dataset import DatasetWriter, read_dataset
from watercube_gb300.fluid import dam_break_params, finalize, snapshot_header
from watercube_gb300.surrogate import Sample


def fnv1a64(data: bytes) -> int:
    h = 14695981039346656037
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def write_snapshot(path, n=64, step=7, seed=3, ids=True):
    p = finalize(dam_break_params(n))
    if ids:
        p.flags |= _abi.WC_FLAG_TRACK_IDS
    h = _abi.SnapshotHeader()
    h.version = 1
    h.header_bytes = C.sizeof(_abi.SnapshotHeader)
    h.num_particles = n
    h.step = step
    h.seed = seed
    h.has_ids = 1 if ids else 0
    h.params = p
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    vel = rng.normal(0, 1, (n, 4)).astype(np.float32)
    head = bytearray(bytes(h))
    head[0:8] = b"WCSNAP\x00\x01"  # (a ctypes char array would stop at the NUL)
    body = bytes(head) + pos.tobytes() + vel.tobytes()
    if ids:
        body += rng.permutation(n).astype(np.uint32).tobytes()
    data = body + struct.pack("<Q", fnv1a64(body))
    path.write_bytes(data)
    return data


def test_snapshot_header_reader(wclib, tmp_path):
    f = tmp_path / "a.wcsnap"
    write_snapshot(f)
    h = snapshot_header(f)
    assert h.num_particles == 64 and h.step == 7 and h.seed == 3 and h.has_ids == 1
    assert h.params.num_particles == 64


@pytest.mark.parametrize("damage", ["flip_body", "flip_checksum", "magic", "truncate", "trailing", "version"])
def test_snapshot_reader_rejects_damage(wclib, tmp_path, damage):
    f = tmp_path / "b.wcsnap"
    data = bytearray(write_snapshot(f, ids=False))
    if damage == "flip_body":
        data[C.sizeof(_abi.SnapshotHeader) + 5] ^= 0x10
    elif damage == "flip_checksum":
        data[-1] ^= 1
    elif damage == "magic":
        data[0:1] = b"X"
    elif damage == "truncate":
        data = data[:-9]
    elif damage == "trailing":
        data += b"\x00"
    elif damage == "version":
        data[8] = 2
    f.write_bytes(bytes(data))
    with pytest.raises(_abi.WatercubeError) as e:
        snapshot_header(f)
    assert e.value.args[0].startswith("[status 1]") or "snapshot" in str(e.value)


def test_snapshot_reader_missing_file(wclib, tmp_path):
    with pytest.raises(_abi.WatercubeError):
        snapshot_header(tmp_path / "none.wcsnap")


def samples(seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for scene, n in ((0, 50), (1, 33), (0, 50)):
        st = np.zeros(n, _abi.PARTICLE_DTYPE)
        st["position"] = rng.uniform(0, 1, (n, 3))
        st["velocity"] = rng.normal(0, 1, (n, 3))
        hist = rng.normal(0, 1, (5, n, 4)).astype(np.float32)
        tgt = rng.normal(0, 9, (n, 4)).astype(np.float32)
        out.append(Sample(scene, len(out), 1e-3, st, hist, tgt))
    return out


def test_dataset_round_trip(wclib, tmp_path):
    params = [finalize(dam_break_params(50)), finalize(dam_break_params(33))]
    f = tmp_path / "d.wcdata"
    sm = samples()
    with DatasetWriter(f, params) as w:
        for s in sm:
            w.write(s)
    back = list(read_dataset(f))
    assert len(back) == len(sm)
    for (p, b), a in zip(back, sm):
        assert bytes(p) == bytes(params[a.scene])
        assert (b.scene, b.step, b.dt) == (a.scene, a.step, np.float32(a.dt))
        assert b.state.tobytes() == a.state.tobytes()
        assert np.array_equal(b.hist, a.hist) and np.array_equal(b.target, a.target)


def test_dataset_detects_corruption(wclib, tmp_path):
    params = [finalize(dam_break_params(50)), finalize(dam_break_params(33))]
    f = tmp_path / "d.wcdata"
    with DatasetWriter(f, params) as w:
        for s in samples():
            w.write(s)
    data = bytearray(f.read_bytes())
    data[-7] ^= 0x40  # inside the last record's target array
    f.write_bytes(bytes(data))
    it = read_dataset(f)
    next(it)
    next(it)
    with pytest.raises(_abi.WatercubeError):
        next(it)
    f.write_bytes(bytes(data[:-3]))
    with pytest.raises(_abi.WatercubeError):
        list(read_dataset(f, verify=False))
