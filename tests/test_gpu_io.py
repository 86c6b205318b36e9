"""UniTensor(fname) / UniTensor::save through the C ABI: files written by the
reference's UniTensor::save load with their bonds, labels and elements;
saving a loaded tensor gives the reference's bytes back; the reference's own
fixtures in its older layout (Swig/examples/egU3_W, egU3_WT, egU1_H_U1, here
rebuilt byte for byte from their decoded contents) load too, and egU3_WT is
egU3_W transposed, bit for bit."""
import json
import os

import numpy as np
import pytest

from oracle import uni10_io

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def tu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from trim_gb300 import uni10 as tu

    tu.set_stream(torch.cuda.current_stream().cuda_stream)
    return tu


def runs(bonds):
    return [[t, [list(r) for r in rr]] for t, rr in bonds]


def test_load_files_the_reference_saved(tu, tmp_path):
    with open(os.path.join(GOLD, "saved.json")) as f:
        index = json.load(f)
    for e in index:
        path = os.path.join(GOLD, "saved", e["file"])
        t = tu.UniTensor.load(path)
        assert runs(t.bonds()) == e["bonds"], e["file"]
        assert t.labels() == e["labels"]
        if e["elem"] is not None:
            assert np.array_equal(t.get_elem(), np.array(e["elem"]))
            out = tmp_path / e["file"]
            t.save(str(out))
            with open(path, "rb") as a, open(out, "rb") as b:
                assert a.read() == b.read(), e["file"]  # the reference's bytes back


def test_load_the_reference_fixtures_in_the_older_layout(tu, tmp_path):
    z = np.load(os.path.join(GOLD, "legacy.npz"))
    meta = json.loads(bytes(z["_meta"]).decode())
    loaded = {}
    for name in ("egU3_W", "egU3_WT", "egU1_H_U1"):
        m = meta[name]
        bonds = [(t, [tuple(r) for r in rr]) for t, rr in m["bonds"]]
        path = tmp_path / name
        path.write_bytes(uni10_io.legacy_bytes(bonds, m["labels"], z[name], m["status"]))
        t = tu.UniTensor.load(str(path))
        assert runs(t.bonds()) == m["bonds"] and t.labels() == m["labels"]
        assert np.array_equal(t.get_elem(), z[name])
        loaded[name] = t
    w = loaded["egU3_W"].copy()
    w.transpose()
    assert np.array_equal(w.get_elem(), z["egU3_WT"])


def test_malformed_file_is_refused(tu, tmp_path):
    from trim_gb300.capi import TnError

    bad = tmp_path / "bad.uni10"
    raw = open(os.path.join(GOLD, "saved", "u1_rank3.uni10"), "rb").read()
    bad.write_bytes(raw[:-5])  # truncated elements
    with pytest.raises(TnError) as e:
        tu.UniTensor.load(str(bad))
    assert e.value.code == 9  # TN_ERR_FILE
