"""Workloads on the GPU against the CPU oracle (FP64, 1e-13) and split
precision against FP64 (1e-12): the Z2 iPEPS CTM quadrant at full size
(chi=128, D=8) and the dense MERA ascend at chi=12 (chi=24 and the full
1024-contraction batch are in test_gpu_full_size.py)."""
import numpy as np
import pytest

from oracle import symtensor as st
from trim_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


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


def test_ipeps_ctm_full_size(tu):
    import bench

    spec = wl.ipeps_ctm()
    dev, els = bench.ipeps_device(tu, spec)
    net = tu.Network(spec["net"])
    for n, t in dev.items():
        net.put_tensor(n, t)
    q64 = net.launch("fp64").get_elem()
    # oracle: the same construction on the CPU
    site, C_, T1, T2 = spec["tensors"]
    a = st.UniTensor(ob(site.bonds), site.labels, els["a"])
    ac = a.copy()
    ac.set_label([0, 11, 12, 13, 14])
    aa = st.contract(a, ac)
    for x in (1, 2, 3, 4):
        aa.combine_bond([x, x + 10])
    aa.permute_rows(2)
    assert np.array_equal(dev["A2"].get_elem(), aa.elem)  # bit-exact double layer (same BLAS-free path? see below)
    aa.set_label([10, 20, 30, 40])
    onet = st.Network(text=spec["net"])
    onet.put_tensor("A2", aa)
    for s in (C_, T1, T2):
        onet.put_tensor(s.name, st.UniTensor(ob(s.bonds), s.labels, els[s.name]))
    qo = onet.launch().elem
    assert rel(q64, qo) <= 1e-13
    qs = net.launch("split").get_elem()
    assert rel(qs, q64) <= 1e-12


def test_mera_chi12_full_network(tu):
    spec = wl.mera(chi=12)
    rng = np.random.default_rng(0)
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    for dname, text in spec["nets"].items():
        net = tu.Network(text)
        keep = [tu.UniTensor(s.bonds, s.labels, els[s.name]) for s in spec["tensors"]]
        for s, t in zip(spec["tensors"], keep):
            net.put_tensor(s.name, t)
        r64 = net.launch("fp64").get_elem()
        onet = st.Network(text=text)
        for s in spec["tensors"]:
            onet.put_tensor(s.name, st.UniTensor(ob(s.bonds), s.labels, els[s.name]))
        assert rel(r64, onet.launch().elem) <= 1e-13, dname
        rs = net.launch("split_tc").get_elem()
        assert rel(rs, r64) <= 1e-12, dname
        m = rs.reshape(144, 144)
        assert np.linalg.norm(m - m.T) / np.linalg.norm(m) <= 1e-12  # Hermiticity preserved
