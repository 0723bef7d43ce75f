"""Server snapshot format, without a GPU: hepem_server_snapshot_check accepts
a snapshot written to the documented layout (include/g4hepem_gb300.h,
csrc/server.cu) and rejects a damaged, truncated or foreign one;
native.snapshot_records reads the records back."""
import struct

import numpy as np
import pytest

from g4hepem_gb300 import native, workload as W


def fnv1a(b: bytes) -> int:
    h = 1469598103934665603
    for x in b:
        h = ((h ^ x) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def write_snapshot(reqs) -> bytes:
    body = bytearray(b"HEPEMSNP" + struct.pack("<II", 1, 0) +
                     struct.pack("<QQ", len(reqs), sum(len(r["state"]["ekin"]) for r in reqs)))
    for r in reqs:
        n = len(r["state"]["ekin"])
        body += struct.pack("<qqQiBBH", r["id"], n, r["seed"], r["steps"], r["admitted"], 0, 0)
        for f, dt in native.STATE_FIELDS:
            body += np.ascontiguousarray(r["state"][f], dtype=dt).tobytes()
        body += r["edep"].astype(np.float64).tobytes() + np.zeros(n, np.float64).tobytes()
        body += np.zeros(n, np.int32).tobytes() + r["tsteps"].astype(np.int32).tobytes()
    return bytes(body) + struct.pack("<Q", fnv1a(bytes(body)))


@pytest.fixture
def snap():
    a = W.mixed_batch(3, seed=1)
    b = W.mixed_batch(5, seed=2)
    return write_snapshot([
        dict(id=7, seed=11, steps=4, admitted=1, state=a, edep=np.array([1.0, 2.0, 3.0]), tsteps=np.full(3, 4)),
        dict(id=9, seed=12, steps=0, admitted=0, state=b, edep=np.zeros(5), tsteps=np.zeros(5)),
    ]), a, b


def test_snapshot_check_and_records(snap):
    s, a, b = snap
    assert native.snapshot_check(s) == (2, 8)
    recs = native.snapshot_records(s)
    assert [(r["id"], r["n"], r["seed"], r["steps"], r["admitted"]) for r in recs] == \
        [(7, 3, 11, 4, True), (9, 5, 12, 0, False)]
    for f, _ in native.STATE_FIELDS:
        assert np.array_equal(recs[0]["state"][f], a[f]) and np.array_equal(recs[1]["state"][f], b[f])
    assert np.array_equal(recs[0]["sums"]["edep"], [1.0, 2.0, 3.0])
    assert np.array_equal(recs[0]["sums"]["track_steps"], [4, 4, 4])


def test_damaged_snapshots_rejected(snap):
    s = snap[0]
    bad = bytearray(s)
    bad[100] ^= 1
    for b in (bytes(bad), s[:-9] + s[-8:], b"HEPEMIMG" + s[8:], s[:20], b""):
        with pytest.raises(native.HepEmError) as e:
            native.snapshot_check(b)
        assert e.value.code == 2  # HEPEM_PARSE_ERROR
    # a record whose size runs past the end: re-checksummed, still rejected
    body = bytearray(s[:-8])
    struct.pack_into("<q", body, 32 + 8, 10 ** 6)
    with pytest.raises(native.HepEmError):
        native.snapshot_check(bytes(body) + struct.pack("<Q", fnv1a(bytes(body))))
