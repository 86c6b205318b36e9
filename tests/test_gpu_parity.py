"""GPU parity: the CUDA path through the C ABI against the reference's golden
outputs and the CPU oracle.  Bit-exact for permute/transpose (pure data
movement); FP64 contraction within 1e-13 relative Frobenius error."""
import hashlib

import numpy as np
import pytest

from oracle import symtensor as st
from tests import golden_data as G
from trim_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-13


@pytest.fixture(scope="module")
def tu():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from trim_gb300 import uni10 as tu

    tu.set_stream(torch.cuda.current_stream().cuda_stream)  # ordered with torch's work on the tensors
    return tu


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def to_obonds(spec_bonds):
    return [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in spec_bonds]


PERM = [c for c in G.cases().values() if c["kind"] == "permute"]
CON = [c for c in G.cases().values() if c["kind"] == "contract"]


@pytest.mark.parametrize("case", PERM, ids=[c["id"] for c in PERM])
def test_permute_transpose_bit_exact(tu, case):
    t = tu.UniTensor(G.bonds_of(case["T"]), case["T"]["labels"], G.arr(case["id"], "T"))
    t.permute(case["new_labels"], case["rownum"])
    assert [[b[0], [list(r) for r in b[1]]] for b in t.bonds()] == case["out"]["bonds"]
    assert t.labels() == case["out"]["labels"]
    assert sha(t.get_elem()) == case["out"]["sha256"]
    t.transpose()
    assert np.array_equal(t.get_elem(), G.arr(case["id"], "PT"))


@pytest.mark.parametrize("case", PERM, ids=[c["id"] for c in PERM])
def test_complex_permute_transpose_ctranspose_bit_exact(tu, case):
    """Complex (cflag) permute, transpose and cTranspose on the GPU
    (UniTensorComplex.cpp:447-825): re = T, im = -2 T (exact) give
    (P, -2 P), then (PT, -2 PT), and conjugated (PT, 2 PT), bit for bit."""
    import torch

    bonds = G.bonds_of(case["T"])
    labels, new = case["T"]["labels"], case["new_labels"]
    rsp = [labels.index(l) for l in new]
    out = [wl.change(bonds[rsp[b]], 1 if b < case["rownum"] else -1) for b in range(len(bonds))]
    x = G.arr(case["id"], "T")
    z = torch.from_numpy(x + 1j * (-2.0 * x)).cuda()
    y = torch.full_like(z, complex(np.nan, np.nan))
    torch.cuda.synchronize()  # the library runs on its own stream
    src, dst = tu.SectorMap(bonds), tu.SectorMap(out)
    tu.permute_device_c128(src, dst, rsp, z.data_ptr(), y.data_ptr())
    tu.sync()
    p, pt = G.arr(case["id"], "P"), G.arr(case["id"], "PT")
    got = y.cpu().numpy()
    assert np.array_equal(got.real, p) and np.array_equal(got.imag, -2.0 * p)
    tmap = tu.SectorMap(G.bonds_of(case["out_transpose"]))
    for conj in (False, True):
        w = torch.full_like(z, complex(np.nan, np.nan))
        torch.cuda.synchronize()
        tu.transpose_device_c128(dst, tmap, conj, y.data_ptr(), w.data_ptr())
        tu.sync()
        got = w.cpu().numpy()
        assert np.array_equal(got.real, pt)
        assert np.array_equal(got.imag, (2.0 if conj else -2.0) * pt)


@pytest.mark.parametrize("perm,rn", [((4, 5, 0, 1, 2, 3), 2), ((0, 3, 5, 1, 2, 4), 3), ((1, 2, 0, 3, 4, 5), 3),
                                     ((5, 4, 3, 2, 1, 0), 3), ((0, 1, 2, 3, 5, 4), 3)])
def test_complex_dense_permutes_bit_exact(tu, perm, rn):
    """Dense rank-6 chi=12 complex permutes (2-D transpose, stacked planes,
    long rows) against torch's permute."""
    import torch

    chi = 12
    bonds = [wl.dense_bond(1, chi)] * 3 + [wl.dense_bond(-1, chi)] * 3
    g = torch.Generator(device="cuda").manual_seed(11)
    x = torch.randn(chi ** 6, dtype=torch.complex128, device="cuda", generator=g)
    y = torch.empty_like(x)
    out = [wl.change(bonds[perm[b]], 1 if b < rn else -1) for b in range(6)]
    torch.cuda.synchronize()  # the library runs on its own stream
    tu.permute_device_c128(tu.SectorMap(bonds), tu.SectorMap(out), list(perm), x.data_ptr(), y.data_ptr())
    tu.sync()
    assert torch.equal(y, x.view([chi] * 6).permute(*perm).reshape(-1))


FGATE = [c for c in G.cases().values() if c["kind"] == "addgate"]
FNET = [c for c in G.cases().values() if c["kind"] == "fnet"]


@pytest.mark.parametrize("case", FGATE, ids=[c["id"] for c in FGATE])
def test_add_gate_bit_exact(tu, case):
    t = tu.UniTensor(G.bonds_of(case["T"]), case["T"]["labels"], G.arr(case["id"], "T"))
    t.add_gate([tuple(p) for p in case["swaps"]])
    assert np.array_equal(t.get_elem(), G.arr(case["id"], "G"))


@pytest.mark.parametrize("case", FGATE, ids=[c["id"] for c in FGATE])
def test_add_gate_c128_bit_exact(tu, case):
    """Complex addGate (UniTensorComplex.cpp:927-980): re = T, im = -2 T
    give (G, -2 G) bit for bit."""
    import torch

    x = G.arr(case["id"], "T")
    z = torch.from_numpy(x + 1j * (-2.0 * x)).cuda()
    torch.cuda.synchronize()
    tu.add_gate_c128(tu.SectorMap(G.bonds_of(case["T"])), [tuple(p) for p in case["swaps"]], z.data_ptr())
    tu.sync()
    g, got = G.arr(case["id"], "G"), z.cpu().numpy()
    assert np.array_equal(got.real, g) and np.array_equal(got.imag, -2.0 * g)


def _fnet(tu, case):
    net = tu.Network(case["net"])
    ts = {}
    for name, meta in case["tensors"].items():
        ts[name] = tu.UniTensor(G.bonds_of(meta), meta["labels"], G.arr(case["id"], name))
        net.put_tensor(name, ts[name])
    return net, ts


@pytest.mark.parametrize("case", FNET, ids=[c["id"] for c in FNET])
def test_fermionic_network_swap_gates(tu, case):
    """Network::launch on fermionic tensors puts the swap gates of its
    contraction order on the tensors once (Network.cpp:697-717, 944-993):
    the result matches the reference, a second launch does not apply them
    again, and a tensor put anew gets them again."""
    ref = G.arr(case["id"], "R")
    net, ts = _fnet(tu, case)
    for _ in range(2):
        r = net.launch("fp64")
        assert [[b[0], [list(x) for x in b[1]]] for b in r.bonds()] == case["R"]["bonds"]
        assert r.labels() == case["R"]["labels"]
        assert rel(r.get_elem(), ref) <= FP64_TOL
    for name in case["tensors"]:
        net.put_tensor(name, ts[name])
        assert rel(net.launch("fp64").get_elem(), ref) <= FP64_TOL


def test_fermionic_network_with_gates_refuses_capture(tu):
    from trim_gb300 import capi

    for case in FNET:
        net, _ = _fnet(tu, case)
        ref = net.launch("fp64").get_elem()
        try:
            net.capture("fp64")
        except capi.TnError as e:
            assert e.code == 7  # TN_ERR_UNSUPPORTED
            assert "swap gates" in str(e)
            return
        net.replay()  # no gate on any tensor: capture is allowed
        assert rel(net.output().get_elem(), ref) <= FP64_TOL
    pytest.fail("no fixture carries a swap gate")


@pytest.mark.parametrize("case", CON, ids=[c["id"] for c in CON])
def test_contract_fp64(tu, case):
    a = tu.UniTensor(G.bonds_of(case["A"]), case["A"]["labels"], G.arr(case["id"], "A"))
    b = tu.UniTensor(G.bonds_of(case["B"]), case["B"]["labels"], G.arr(case["id"], "B"))
    c = tu.contract(a, b, fast=False, mode="fp64")
    assert [[x[0], [list(r) for r in x[1]]] for x in c.bonds()] == case["out"]["bonds"]
    assert c.labels() == case["out"]["labels"]
    assert rel(c.get_elem(), G.arr(case["id"], "C")) <= FP64_TOL
    # fast=false restores the operands bit for bit
    assert np.array_equal(a.get_elem(), G.arr(case["id"], "A"))
    assert a.labels() == case["A"]["labels"]


def test_contract_output_blocks_without_sectors_are_zero(tu):
    """A[x|k] . B[k|y] where k carries charges A's rows reach but B's columns
    do not: output blocks with no sector GEMM stay zero, as the reference's
    zero-filled result does; the other blocks match the oracle."""
    x = wl.u1_bond(1, (-1, 0, 1), (2, 3, 2))
    k = wl.u1_bond(-1, (-1, 0), (1, 2))  # no charge 1: output block 1 has no sector
    y = wl.u1_bond(-1, (0, 1), (2, 3))
    a_bonds, b_bonds = [x, k], [wl.change(k, 1), y]
    rng = np.random.default_rng(31)
    ea = rng.uniform(-1, 1, wl.elem_count(a_bonds))
    eb = rng.uniform(-1, 1, wl.elem_count(b_bonds))
    la, lb = [1, 2], [2, 3]
    for fused in (False, True):  # with and without an operand permute in front
        a = tu.UniTensor(a_bonds, la, ea)
        b = tu.UniTensor(b_bonds, lb, eb)
        if fused:
            a.permute([2, 1], 1)  # the contraction permutes it back (a view)
        c = tu.contract(a, b, fast=False, mode="fp64")
        oa = st.UniTensor(to_obonds(a_bonds), la, ea)
        if fused:
            oa.permute([2, 1], 1)
        ob = st.UniTensor(to_obonds(b_bonds), lb, eb)
        oc = st.contract(oa, ob)
        assert c.labels() == oc.labels
        assert rel(c.get_elem(), oc.elem) <= FP64_TOL
        assert np.count_nonzero(oc.elem == 0.0) > 0  # the case has a block without a sector


def test_workload1_permute_and_contract(tu):
    c = G.cases()["u1_rank4"]
    spec = wl.u1_rank4()
    A, B = spec["tensors"]
    ta = tu.UniTensor(A.bonds, A.labels, G.arr("u1_rank4", "A"))
    tb = tu.UniTensor(B.bonds, B.labels, G.arr("u1_rank4", "B"))
    ta.permute([0, 1, 3, 2], 2)
    assert sha(ta.get_elem()) == c["PA"]["sha256"]
    tc = tu.contract(ta, tb, mode="fp64")
    assert rel(tc.get_elem(), G.arr("u1_rank4", "C")) <= FP64_TOL


def _itebd_inputs():
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    return spec, {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}


def test_itebd_network_fp64(tu):
    c = G.cases()["itebd"]
    spec, els = _itebd_inputs()
    assert {k: sha(v) for k, v in els.items()} == c["inputs_sha"]
    net = tu.Network(spec["net"])
    ts = {}
    for s in spec["tensors"]:
        ts[s.name] = tu.UniTensor(s.bonds, s.labels, els[s.name])
        net.put_tensor(s.name, ts[s.name])
    th = net.launch(mode="fp64")
    assert [[x[0], [list(r) for r in x[1]]] for x in th.bonds()] == c["TH"]["bonds"]
    assert th.labels() == c["TH"]["labels"]
    assert rel(th.get_elem(), G.arr("itebd", "TH")) <= FP64_TOL
    assert net.tree() == "(((((La A) Lb) B) Lc) U)"


def test_greedy_network_tree_and_values(tu):
    c = G.cases()["greedy_net"]
    net = tu.Network(c["net"])
    keep = []
    for n, meta in c["tensors"].items():
        t = tu.UniTensor(G.bonds_of(meta), meta["labels"], G.arr("greedy_net", n))
        keep.append(t)
        net.put_tensor(n, t)
    onet = st.Network(text=c["net"])
    for n, meta in c["tensors"].items():
        onet.put_tensor(n, st.UniTensor(to_obonds(G.bonds_of(meta)), meta["labels"], G.arr("greedy_net", n)))
    r = net.launch(mode="fp64")
    assert rel(r.get_elem(), G.arr("greedy_net", "R")) <= FP64_TOL


def test_batched_small_fp64(tu):
    c = G.cases()["batched_small"]
    spec = wl.batched(**c["params"])
    for i, (t1, t2) in enumerate(spec["pairs"]):
        a = tu.UniTensor(t1.bonds, t1.labels, G.arr("batched_small", t1.name))
        b = tu.UniTensor(t2.bonds, t2.labels, G.arr("batched_small", t2.name))
        r = tu.contract(a, b, mode="fp64")
        assert rel(r.get_elem(), G.arr("batched_small", f"C{i}")) <= FP64_TOL


def test_mera_small_fp64(tu):
    c = G.cases()["mera_small"]
    spec = wl.mera(**c["params"])
    rng = np.random.default_rng(0)
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    for dname, netx in spec["nets"].items():
        net = tu.Network(netx)
        keep = []
        for s in spec["tensors"]:
            t = tu.UniTensor(s.bonds, s.labels, els[s.name])
            keep.append(t)
            net.put_tensor(s.name, t)
        r = net.launch(mode="fp64")
        assert rel(r.get_elem(), G.arr("mera_small", dname)) <= FP64_TOL


def test_ipeps_small_double_layer_and_quadrant(tu):
    c = G.cases()["ipeps_small"]
    spec = wl.ipeps_ctm(**c["params"])
    site, C_, T1, T2 = spec["tensors"]
    a = tu.UniTensor(site.bonds, site.labels, G.arr("ipeps_small", "a"))
    ac = a.copy()
    ac.set_label([0, 11, 12, 13, 14])
    aa = tu.contract(a, ac, mode="fp64")
    for x in (1, 2, 3, 4):
        aa.combine_bond([x, x + 10])
    aa.permute(aa.labels(), 2)
    assert [[x[0], [list(r) for r in x[1]]] for x in aa.bonds()] == c["AA"]["bonds"]
    assert rel(aa.get_elem(), G.arr("ipeps_small", "AA")) <= FP64_TOL
    aa.set_label([10, 20, 30, 40])
    net = tu.Network(spec["net"])
    keep = [aa]
    for s in (C_, T1, T2):
        t = tu.UniTensor(s.bonds, s.labels, G.arr("ipeps_small", s.name))
        keep.append(t)
        net.put_tensor(s.name, t)
    net.put_tensor("A2", aa)
    q = net.launch(mode="fp64")
    assert rel(q.get_elem(), G.arr("ipeps_small", "Q")) <= FP64_TOL


def test_large_dense_permute_bit_exact(tu):
    """A chi=20 rank-6 dense tensor (64M elements): the transpose-mode tiles."""
    chi = 20
    bonds = [wl.dense_bond(1, chi)] * 3 + [wl.dense_bond(-1, chi)] * 3
    rng = np.random.default_rng(3)
    x = rng.standard_normal(chi ** 6)
    t = tu.UniTensor(bonds, list(range(6)), x)
    t.permute([4, 5, 0, 1, 2, 3], 2)
    want = x.reshape([chi] * 6).transpose(4, 5, 0, 1, 2, 3).ravel()
    assert np.array_equal(t.get_elem(), want)
    t.permute([2, 0, 5, 4, 1, 3], 3)  # labels now (4,5,0,1,2,3) -> arbitrary order
    want2 = want.reshape([chi] * 6)
    cur = [4, 5, 0, 1, 2, 3]
    want2 = want2.transpose([cur.index(l) for l in [2, 0, 5, 4, 1, 3]]).ravel()
    assert np.array_equal(t.get_elem(), want2)


def test_dense_permutes_with_short_contiguous_bonds_bit_exact(tu):
    """The MERA ascend's permutes where both the destination- and the
    source-contiguous bond are short (chi = 12 here): transpose tiles of
    several stacked planes, ragged in every direction (chi = 13)."""
    for chi in (12, 13):
        bonds = [wl.dense_bond(1, chi)] * 3 + [wl.dense_bond(-1, chi)] * 3
        rng = np.random.default_rng(chi)
        x = rng.standard_normal(chi ** 6)
        for perm, rn in (((0, 3, 5, 1, 2, 4), 3), ((1, 2, 3, 5, 0, 4), 4), ((2, 3, 5, 0, 1, 4), 3),
                         ((0, 2, 3, 5, 1, 4), 4), ((3, 5, 0, 1, 2, 4), 2)):
            t = tu.UniTensor(bonds, list(range(6)), x)
            t.permute(list(perm), rn)
            want = x.reshape([chi] * 6).transpose(perm).ravel()
            assert np.array_equal(t.get_elem(), want), (chi, perm)


def test_errors_on_device_path(tu):
    from trim_gb300 import capi

    a = tu.UniTensor([wl.dense_bond(1, 3), wl.dense_bond(-1, 4)], [1, 2], np.ones(12))
    b = tu.UniTensor([wl.dense_bond(1, 5), wl.dense_bond(-1, 4)], [2, 3], np.ones(20))
    with pytest.raises(capi.TnError) as e:
        tu.contract(a, b)
    assert "Cannot contract two bonds having different dimensions" in str(e.value)
    with pytest.raises(capi.TnError) as e:
        a.permute([1, 9], 1)
    assert "do not 1-1 correspond" in str(e.value)


def test_ipeps_short_row_permute_bit_exact(tu):
    """The iPEPS quadrant's operand permute X[10,3|4,20] -> [3,4|10,20] at
    chi=32, D=4 (rows of 2-4 elements stacked into 3-D tiles): bit-exact
    against the oracle, real and complex."""
    import torch

    rng = np.random.default_rng(19)
    spec = wl.ipeps_ctm(chi=32, D=4)
    c_in, dd, c_out = spec["tensors"][2].bonds
    bonds = [dd, wl.change(c_in, 1), wl.change(c_out, -1), wl.change(dd, -1)]
    labels, new, rn = [10, 3, 4, 20], [3, 4, 10, 20], 2
    x = rng.uniform(-1, 1, wl.elem_count(bonds))
    t = tu.UniTensor(bonds, labels, x)
    t.permute(new, rn)
    o = st.UniTensor(to_obonds(bonds), labels, x)
    o.permute(new, rn)
    assert np.array_equal(t.get_elem(), o.elem)
    rsp = [labels.index(l) for l in new]
    out = [wl.change(bonds[rsp[b]], 1 if b < rn else -1) for b in range(4)]
    z = torch.from_numpy(x + 1j * (0.25 * x)).cuda()
    y = torch.empty_like(z)
    torch.cuda.synchronize()
    tu.permute_device_c128(tu.SectorMap(bonds), tu.SectorMap(out), rsp, z.data_ptr(), y.data_ptr())
    tu.sync()
    got = y.cpu().numpy()
    assert np.array_equal(got.real, o.elem) and np.array_equal(got.imag, 0.25 * o.elem)
