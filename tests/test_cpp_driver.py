"""The C++ drop-in boundary: tests/cpp/drop_in_driver.cpp, written against
the reference's API (uni10.hpp), compiles against include/ and links against
libtrim_gb300.so (CPU); on a GPU it runs, and everything it saved in the
reference's binary layout is checked against the oracle: permute bit-exact,
contract and Network::launch within 1e-13, Block::svd / Block::eigh values
within 1e-13 of LAPACK's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import symtensor as st
from oracle import uni10_io

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "trim_gb300", "_lib")
SRC = os.path.join(ROOT, "tests", "cpp", "drop_in_driver.cpp")


def build_driver(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    if not os.path.exists(os.path.join(LIBDIR, "libtrim_gb300.so")):
        pytest.skip("library not built")
    exe = str(tmp_path / "drop_in_driver")
    cmd = ["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), SRC, "-L" + LIBDIR, "-ltrim_gb300",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    return exe


def test_driver_compiles_and_links(tmp_path):
    assert os.access(build_driver(tmp_path), os.X_OK)


def to_tensor(d):
    bonds = [st.Bond.from_runs(t, [(st.Qnum(u, p, f), g) for (u, p, f, g) in runs]) for t, runs in d["bonds"]]
    return st.UniTensor(bonds, d["labels"], d["elem"])


@pytest.mark.gpu
def test_driver_runs_and_matches_oracle(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = build_driver(tmp_path)
    out = tmp_path / "out"
    out.mkdir()
    p = subprocess.run([exe, str(out)], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    rd = lambda n: uni10_io.read_tensor(str(out / n))
    A, B = to_tensor(rd("A.bin")), to_tensor(rd("B.bin"))
    # permute: bit-exact
    pa = A.copy()
    pa.permute([2, 1, 3], 2)
    got = rd("PA.bin")
    assert got["labels"] == pa.labels and np.array_equal(got["elem"], pa.elem)
    # contract and the two-tensor network
    ref = st.contract(A.copy(), B.copy())
    for name in ("AB.bin", "NET.bin"):
        got = rd(name)
        r = ref.copy()
        if name == "NET.bin":
            r.permute([1, 2, 4, 5], 3)
        assert got["labels"] == r.labels
        assert np.linalg.norm(got["elem"] - r.elem) <= 1e-13 * np.linalg.norm(r.elem)
    # Block::svd / Block::eigh of M's charge-0 block
    M = to_tensor(rd("M.bin"))
    blk = M.get_block(st.Qnum(0, 0, 0))
    lines = (out / "blocks.txt").read_text().split("\n")
    s = np.array([float(l.split()[1]) for l in lines if l.startswith("s ")])
    e = np.array([float(l.split()[1]) for l in lines if l.startswith("e ")])
    s_ref = st.block_svd(blk)[1]
    e_ref = st.block_eigh(blk)[0]
    assert np.max(np.abs(s - s_ref)) <= 1e-13 * s_ref.max()
    assert np.max(np.abs(e - e_ref)) <= 1e-13 * np.max(np.abs(e_ref))
