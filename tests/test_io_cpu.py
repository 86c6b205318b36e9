"""The reference's binary tensor layouts: files written by the compiled
reference's UniTensor::save (tests/golden/saved/, seeded inputs listed in
saved.json) decode to their inputs, and the older layout the reference's own
fixtures use is reproduced byte for byte by the writer the GPU tests feed to
the product's reader (pinned by the SHA-256 of the reference's files)."""
import hashlib
import json
import os

import numpy as np

from oracle import uni10_io

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def test_saved_files_decode_to_their_inputs():
    with open(os.path.join(GOLD, "saved.json")) as f:
        index = json.load(f)
    assert len(index) == 4
    for e in index:
        d = uni10_io.read_tensor(os.path.join(GOLD, "saved", e["file"]))
        assert d["rflag"] == 1 and d["cflag"] == 0 and d["name"] == e["name"]
        assert d["labels"] == e["labels"]
        assert [[t, [list(r) for r in runs]] for t, runs in d["bonds"]] == e["bonds"]
        if e["elem"] is None:
            assert d["elem"] is None
        else:
            assert np.array_equal(d["elem"], np.array(e["elem"]))


def test_legacy_writer_reproduces_the_reference_fixture_bytes():
    z = np.load(os.path.join(GOLD, "legacy.npz"))
    meta = json.loads(bytes(z["_meta"]).decode())
    for name in ("egU3_W", "egU3_WT", "egU1_H_U1"):
        m = meta[name]
        bonds = [(t, [tuple(r) for r in runs]) for t, runs in m["bonds"]]
        raw = uni10_io.legacy_bytes(bonds, m["labels"], z[name], m["status"])
        assert hashlib.sha256(raw).hexdigest() == m["sha256"], name
