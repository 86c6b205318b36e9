"""The two largest workloads at their stated sizes on the GPU, against the
CPU oracle.

* Dense ternary MERA ascend, chi = 24 (a 1.9e8-element operator, chi^8-sized
  sector GEMMs): for each of the three diagrams the FP64 GPU result is within
  1e-13 (relative Frobenius) of the oracle's numpy/BLAS restatement of
  Network::launch, the split-precision tensor-core result within 1e-12 of the
  FP64 GPU result, and the ascended operator stays symmetric (Hermitian)
  within 1e-12.
* 1024 independent uneven U(1) contractions (bond dims 16..256, charges
  -4..4): one grouped call in FP64 matches the oracle's per-pair contract()
  within 1e-13 per pair, split precision matches FP64 within 1e-12 per pair.
"""
import numpy as np
import pytest

from oracle import symtensor as st
from trim_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-13
SPLIT_TOL = 1e-12


@pytest.fixture(scope="module")
def tu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from trim_gb300 import uni10 as tu

    tu.set_stream(torch.cuda.current_stream().cuda_stream)
    return tu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def ob(bonds):
    return [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in bonds]


@pytest.fixture(scope="module")
def mera24():
    spec = wl.mera(chi=24)
    rng = np.random.default_rng(0)
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    return spec, els


@pytest.mark.parametrize("diagram", ["left", "center", "right"])
def test_mera_chi24_against_oracle(tu, mera24, diagram):
    spec, els = mera24
    text = spec["nets"][diagram]
    net = tu.Network(text)
    keep = [tu.UniTensor(s.bonds, s.labels, els[s.name]) for s in spec["tensors"]]
    for s, t in zip(spec["tensors"], keep):
        net.put_tensor(s.name, t)
    r64 = net.launch("fp64").get_elem()
    rs = net.launch("split").get_elem()
    keep = None
    onet = st.Network(text=text)
    for s in spec["tensors"]:
        onet.put_tensor(s.name, st.UniTensor(ob(s.bonds), s.labels, els[s.name]))
    ro = onet.launch().elem
    onet = None
    assert r64.size == 24 ** 4
    assert rel(r64, ro) <= FP64_TOL, diagram
    assert rel(rs, r64) <= SPLIT_TOL, diagram
    for v in (r64, rs):
        m = v.reshape(576, 576)
        assert np.linalg.norm(m - m.T) / np.linalg.norm(m) <= 1e-12  # Hermiticity preserved


def test_batched_1024_against_oracle(tu):
    spec = wl.batched(n=1024)
    assert len(spec["pairs"]) == 1024
    rng = np.random.default_rng(spec["seed"])
    A, B, oracle_out = [], [], []
    nsec = 0
    for t1, t2 in spec["pairs"]:
        e1, e2 = wl.gen_elems(t1, rng), wl.gen_elems(t2, rng)
        A.append(tu.UniTensor(t1.bonds, t1.labels, e1))
        B.append(tu.UniTensor(t2.bonds, t2.labels, e2))
        oa = st.UniTensor(ob(t1.bonds), t1.labels, e1)
        obb = st.UniTensor(ob(t2.bonds), t2.labels, e2)
        nsec += len(st.sector_gemms(oa, obb))
        oracle_out.append(st.contract(oa, obb).elem)
    assert nsec > 4000  # thousands of sector GEMMs of sizes 1..256
    f64 = [o.get_elem() for o in tu.contract_batch(A, B, "fp64")]
    spl = [o.get_elem() for o in tu.contract_batch(A, B, "split")]
    worst64 = max(rel(g, w) for g, w in zip(f64, oracle_out))
    worst_split = max(rel(g, w) for g, w in zip(spl, f64))
    assert worst64 <= FP64_TOL, worst64
    assert worst_split <= SPLIT_TOL, worst_split
