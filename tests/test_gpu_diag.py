"""Diagonal tensors on the GPU: a tensor built by putBlock with diagonal
matrices contracts as a row or column scale of the other operand (RDotR's
diagRowMul / diagColMul, BlockTools.cpp:45-60, on every block in one launch)
instead of sector GEMMs.  The result must equal the dense sector-GEMM result
on the same values bit for bit (a sum with one non-zero term, rounded once)
and the oracle within 1e-15; the iTEBD network with diagonal Lambdas must
match the dense network and run only the A.B and gate GEMMs."""
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


def ob(bonds):
    return [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in bonds]


def diag_device(tu, spec, elems):
    t = tu.UniTensor(spec.bonds, spec.labels)
    for q, r, c, d in wl.diag_blocks(spec.bonds, elems):
        t.put_block(q, (r, c, d), diag=True)
    return t


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_diagonal_flag(tu):
    spec = wl.itebd()
    La = spec["tensors"][0]
    e = wl.gen_elems(La, np.random.default_rng(0))
    t = diag_device(tu, La, e)
    assert t.is_diagonal() and np.array_equal(t.get_elem(), e)
    assert t.copy().is_diagonal()
    t.set_elem(e)
    assert not t.is_diagonal()  # a dense write
    A = tu.UniTensor(spec["tensors"][1].bonds, spec["tensors"][1].labels)
    assert not A.is_diagonal()  # three bonds


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_itebd_network_with_diagonal_lambdas(tu, mode):
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    dense, diag = tu.Network(spec["net"]), tu.Network(spec["net"])
    keep = []
    for s in spec["tensors"]:
        td = tu.UniTensor(s.bonds, s.labels, els[s.name])
        tg = diag_device(tu, s, els[s.name]) if s.kind == "diag" else td
        keep += [td, tg]
        dense.put_tensor(s.name, td)
        diag.put_tensor(s.name, tg)
    want = dense.launch("fp64").get_elem()
    diag.launch(mode)  # the first split launch times the route candidates
    tu.prof_enable(True)
    got = diag.launch(mode).get_elem()
    prof = tu.prof_read()
    tu.prof_enable(False)
    assert np.array_equal(got, want)  # bit-identical to the dense Lambda GEMMs
    assert prof["diag_scale"]["launches"] == 3
    gemm_flops = sum(v["flops"] for k, v in prof.items() if "gemm" in k)
    assert gemm_flops < 0.4 * 31666456  # only A.B and the gate remain GEMMs
    # the oracle with the same diagonal tensors
    onet = st.Network(text=spec["net"])
    for s in spec["tensors"]:
        t = st.UniTensor(ob(s.bonds), s.labels, els[s.name])
        if s.kind == "diag":
            t = st.UniTensor(ob(s.bonds), s.labels)
            for q, r, c, d in wl.diag_blocks(s.bonds, els[s.name]):
                t.put_block(st.Qnum(*q), d, diag=True, fresh=True)
        onet.put_tensor(s.name, t)
    assert rel(got, onet.launch().elem) <= 1e-15


def test_itebd_graph_with_diagonal_lambdas(tu):
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    net = tu.Network(spec["net"])
    keep = [diag_device(tu, s, els[s.name]) if s.kind == "diag" else tu.UniTensor(s.bonds, s.labels, els[s.name])
            for s in spec["tensors"]]
    for s, t in zip(spec["tensors"], keep):
        net.put_tensor(s.name, t)
    eager = net.launch("fp64").get_elem()
    net.capture("fp64")
    net.replay()
    tu.sync()
    assert np.array_equal(net.output().get_elem(), eager)


@pytest.mark.parametrize("fast", [False, True])
def test_contract_with_diagonal_operand_either_side(tu, fast):
    spec = wl.itebd()
    rng = np.random.default_rng(7)
    La, A, Lb = spec["tensors"][0], spec["tensors"][1], spec["tensors"][2]
    el, ea, eb = wl.gen_elems(La, rng), wl.gen_elems(A, rng), wl.gen_elems(Lb, rng)
    # left: La[-1|10] . A[10,1|11] (row scale of A permuted to (10|1,11))
    la, a = diag_device(tu, La, el), tu.UniTensor(A.bonds, A.labels, ea)
    got = tu.contract(la, a, fast=fast).get_elem()
    want = tu.contract(tu.UniTensor(La.bonds, La.labels, el), tu.UniTensor(A.bonds, A.labels, ea)).get_elem()
    assert np.array_equal(got, want)
    if not fast:  # the operands are restored
        assert la.labels() == La.labels and a.labels() == A.labels
        assert np.array_equal(a.get_elem(), ea)
    # right: A[10,1|11] . Lb[11|12] (column scale)
    a2, lb = tu.UniTensor(A.bonds, A.labels, ea), diag_device(tu, Lb, eb)
    got = tu.contract(a2, lb, fast=fast).get_elem()
    want = tu.contract(tu.UniTensor(A.bonds, A.labels, ea), tu.UniTensor(Lb.bonds, Lb.labels, eb)).get_elem()
    assert np.array_equal(got, want)


def test_rectangular_diagonal_blocks(tu):
    # Lambda[x | y]: x has charges (-1, 0, 1) x (2, 5, 1), y (-1, 0, 1) x (3, 3, 2):
    # blocks 2x3, 5x3, 1x2 with min(R, C) diagonal entries; rows (columns) past
    # the diagonal are zero in the product
    bx = (1, [(-1, 0, 0, 2), (0, 0, 0, 5), (1, 0, 0, 1)])
    by = (-1, [(-1, 0, 0, 3), (0, 0, 0, 3), (1, 0, 0, 2)])
    rng = np.random.default_rng(3)
    lam = tu.UniTensor([bx, by], [1, 2])
    olam = st.UniTensor(ob([bx, by]), [1, 2])
    for q, r, c in wl.block_shapes([bx, by]):
        d = rng.uniform(0.5, 2.0, min(r, c))
        lam.put_block(q, (r, c, d), diag=True)
        olam.put_block(st.Qnum(*q), d, diag=True, fresh=True)
    assert lam.is_diagonal()
    byin = (1, by[1])  # the same charges, incoming (a bond joins an OUT leg to an IN leg)
    bz = (-1, [(-1, 0, 0, 4), (0, 0, 0, 2), (1, 0, 0, 3)])
    ex = rng.standard_normal(wl.elem_count([byin, bz]))
    x = tu.UniTensor([byin, bz], [2, 3], ex)
    got = tu.contract(lam, x).get_elem()
    want = st.contract(olam, st.UniTensor(ob([byin, bz]), [2, 3], ex)).elem
    assert np.array_equal(got, want)
    dense = tu.UniTensor([bx, by], [1, 2], lam.copy().get_elem())
    assert np.array_equal(got, tu.contract(dense, tu.UniTensor([byin, bz], [2, 3], ex)).get_elem())
