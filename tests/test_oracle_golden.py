"""Pins the CPU oracle (oracle/symtensor.py) against the reference's own
outputs (golden fixtures made by the compiled reference) and against the
reference's fixtures.  CPU only."""
import hashlib

import numpy as np
import pytest

from oracle import symtensor as st
from tests import golden_data as G
from trim_gb300 import workloads as wl


def to_bonds(spec_bonds):
    return [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in spec_bonds]


def bonds_meta(t):
    return [[b.type, [[q.u1, q.prt, q.prtf, d] for q, d in zip(b.qnums, b.qdegs)]] for b in t.bonds]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


PERM = [c for c in G.cases().values() if c["kind"] == "permute"]
CON = [c for c in G.cases().values() if c["kind"] == "contract"]


@pytest.mark.parametrize("case", PERM, ids=[c["id"] for c in PERM])
def test_permute_bit_exact(case):
    t = st.UniTensor(to_bonds(G.bonds_of(case["T"])), case["T"]["labels"], G.arr(case["id"], "T"))
    t.permute(case["new_labels"], case["rownum"])
    assert bonds_meta(t) == case["out"]["bonds"]
    assert t.labels == case["out"]["labels"]
    assert sha(t.elem) == case["out"]["sha256"]
    t.transpose()
    assert bonds_meta(t) == case["out_transpose"]["bonds"]
    assert np.array_equal(t.elem, G.arr(case["id"], "PT"))


@pytest.mark.parametrize("case", CON, ids=[c["id"] for c in CON])
def test_contract(case):
    a = st.UniTensor(to_bonds(G.bonds_of(case["A"])), case["A"]["labels"], G.arr(case["id"], "A"))
    b = st.UniTensor(to_bonds(G.bonds_of(case["B"])), case["B"]["labels"], G.arr(case["id"], "B"))
    c = st.contract(a, b)
    ref = G.arr(case["id"], "C")
    assert bonds_meta(c) == case["out"]["bonds"]
    assert c.labels == case["out"]["labels"]
    assert np.linalg.norm(c.elem - ref) <= 1e-13 * max(np.linalg.norm(ref), 1e-300)
    # contract(fast=false) restores the operands
    assert np.array_equal(a.elem, G.arr(case["id"], "A"))


def test_workload1():
    c = G.cases()["u1_rank4"]
    spec = wl.u1_rank4()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    assert {k: sha(v) for k, v in els.items()} == c["inputs_sha"]
    T = {s.name: st.UniTensor(to_bonds(s.bonds), s.labels, els[s.name]) for s in spec["tensors"]}
    T["A"].permute([0, 1, 3, 2], 2)
    assert sha(T["A"].elem) == c["PA"]["sha256"]
    C = st.contract(T["A"], T["B"])
    ref = G.arr("u1_rank4", "C")
    assert np.linalg.norm(C.elem - ref) <= 1e-13 * np.linalg.norm(ref)
    assert sum(2 * m * n * k for m, n, k in st.sector_gemms(T["A"], T["B"])) == 147520


def test_itebd_network_and_svd():
    c = G.cases()["itebd"]
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    assert {k: sha(v) for k, v in els.items()} == c["inputs_sha"]
    net = st.Network(text=spec["net"])
    for s in spec["tensors"]:
        net.put_tensor(s.name, st.UniTensor(to_bonds(s.bonds), s.labels, els[s.name]))
    th = net.launch()
    ref = G.arr("itebd", "TH")
    assert bonds_meta(th) == c["TH"]["bonds"] and th.labels == c["TH"]["labels"]
    assert np.linalg.norm(th.elem - ref) <= 1e-13 * np.linalg.norm(ref)
    sv = np.concatenate([st.block_svd(th.get_block(q))[1] for q in th.block_qnums()])
    sref = G.arr("itebd", "S")
    assert np.max(np.abs(sv - sref)) <= 1e-13 * sref.max()


def test_network_greedy_planner_bit_exact():
    c = G.cases()["greedy_net"]
    net = st.Network(text=c["net"])
    for n, meta in c["tensors"].items():
        net.put_tensor(n, st.UniTensor(to_bonds(G.bonds_of(meta)), meta["labels"], G.arr("greedy_net", n)))
    r = net.launch()
    # identical tree => identical BLAS calls => identical bits
    assert sha(r.elem) == c["R"]["sha256"]


def test_ipeps_small():
    c = G.cases()["ipeps_small"]
    spec = wl.ipeps_ctm(**c["params"])
    site, C, T1, T2 = spec["tensors"]
    a = st.UniTensor(to_bonds(site.bonds), site.labels, G.arr("ipeps_small", "a"))
    ac = a.copy()
    ac.set_label([0, 11, 12, 13, 14])
    aa = st.contract(a, ac)
    for x in (1, 2, 3, 4):
        aa.combine_bond([x, x + 10])
    aa.permute_rows(2)
    assert bonds_meta(aa) == c["AA"]["bonds"]
    assert sha(aa.elem) == c["AA"]["sha256"]
    aa.set_label([10, 20, 30, 40])
    net = st.Network(text=spec["net"])
    for s in (C, T1, T2):
        net.put_tensor(s.name, st.UniTensor(to_bonds(s.bonds), s.labels, G.arr("ipeps_small", s.name)))
    net.put_tensor("A2", aa)
    q = net.launch()
    ref = G.arr("ipeps_small", "Q")
    assert np.linalg.norm(q.elem - ref) <= 1e-13 * np.linalg.norm(ref)


def test_batched_small():
    c = G.cases()["batched_small"]
    spec = wl.batched(**c["params"])
    for i, (t1, t2) in enumerate(spec["pairs"]):
        a = st.UniTensor(to_bonds(t1.bonds), t1.labels, G.arr("batched_small", t1.name))
        b = st.UniTensor(to_bonds(t2.bonds), t2.labels, G.arr("batched_small", t2.name))
        r = st.contract(a, b)
        ref = G.arr("batched_small", f"C{i}")
        assert bonds_meta(r) == c["outs"][f"C{i}"]["bonds"]
        assert np.linalg.norm(r.elem - ref) <= 1e-13 * np.linalg.norm(ref)


def test_mera_small():
    c = G.cases()["mera_small"]
    spec = wl.mera(**c["params"])
    rng = np.random.default_rng(0)
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    for dname, netx in spec["nets"].items():
        net = st.Network(text=netx)
        for s in spec["tensors"]:
            net.put_tensor(s.name, st.UniTensor(to_bonds(s.bonds), s.labels, els[s.name]))
        r = net.launch()
        ref = G.arr("mera_small", dname)
        assert np.linalg.norm(r.elem - ref) <= 1e-13 * np.linalg.norm(ref)
        # the ascended operator of a symmetric operator is symmetric
        m = r.get_block(r.block_qnums()[0])
        assert np.linalg.norm(m - m.T) <= 1e-13 * np.linalg.norm(m)


def test_legacy_fixture_transpose_known_answer():
    """egU3_WT is egU3_W.transpose() saved by the reference: its elements are
    a permutation of W's, reproduced bit-exactly."""
    L = G.legacy()
    mw = L["_meta"]["egU3_W"]
    w = st.UniTensor(to_bonds(G.bonds_of(mw)), mw["labels"], L["egU3_W"])
    w.transpose()
    assert bonds_meta(w) == L["_meta"]["egU3_WT"]["bonds"]
    assert np.array_equal(w.elem, L["egU3_WT"])


def test_legacy_fixture_svd():
    """mat_U (4x4), mat_Sigma (4), mat_VT (4x5): the reference's SVD factors.
    Re-factorising U.S.VT gives back S."""
    L = G.legacy()
    u, s, vt = L["mat_U"].reshape(4, 4), L["mat_Sigma"], L["mat_VT"].reshape(4, 5)
    m = (u * s) @ vt
    _, s2, _ = st.block_svd(m)
    assert np.allclose(s2, s, rtol=1e-13, atol=1e-15)


def test_sector_map_edge_cases():
    # no OUT bonds: one column per block (UniTensorReal.cpp:1276-1282)
    t = st.UniTensor(to_bonds([(1, [(1, 0, 0, 2), (-1, 0, 0, 1)]), (1, [(-1, 0, 0, 1), (1, 0, 0, 1)])]))
    assert [(b[0].u1, b[1], b[2]) for b in t.smap.blocks] == [(0, 3, 1)]
    # IN after OUT is rejected
    with pytest.raises(ValueError):
        st.UniTensor(to_bonds([(-1, [(0, 0, 0, 2)]), (1, [(0, 0, 0, 2)])]))
    # no common charge -> no block
    with pytest.raises(ValueError):
        st.UniTensor(to_bonds([(1, [(1, 0, 0, 2)]), (-1, [(0, 0, 0, 2)])]))


@pytest.mark.parametrize("case_id", ["eigh0", "eigh1", "eigh2"])
def test_eigh_oracle_matches_reference(case_id):
    """Block::eigh (dsyev on the lower triangle) of the compiled reference:
    the restatement gives its eigenvalues and eigenvector projectors.  The
    inputs of eigh0/eigh1 are not symmetric, so this also pins the triangle."""
    from tests.eigh_check import check_eigh, golden_eigh_blocks

    for a, e_ref, v_ref in golden_eigh_blocks(case_id):
        e, v = st.block_eigh(a)
        check_eigh(a, e, v, e_ref, v_ref)
        # the other triangle gives a different spectrum whenever a is not symmetric
        if not np.array_equal(a, a.T):
            e_up = np.linalg.eigvalsh(np.triu(a) + np.triu(a, 1).T)
            assert np.max(np.abs(e_up - e_ref)) > 1e-6


FGATE = [c for c in G.cases().values() if c["kind"] == "addgate"]
FNET = [c for c in G.cases().values() if c["kind"] == "fnet"]


@pytest.mark.parametrize("case", FGATE, ids=[c["id"] for c in FGATE])
def test_add_gate_bit_exact(case):
    t = st.UniTensor(to_bonds(G.bonds_of(case["T"])), case["T"]["labels"], G.arr(case["id"], "T").copy())
    st.add_gate(t, [tuple(p) for p in case["swaps"]])
    assert np.array_equal(t.elem, G.arr(case["id"], "G"))


@pytest.mark.parametrize("case", FNET, ids=[c["id"] for c in FNET])
def test_fermionic_network_swap_gates(case):
    """Network::launch with swap gates on fermionic tensors: the restated
    addSwap/addGate reproduce the reference within 1e-13 (identical BLAS)."""
    net = st.Network(text=case["net"])
    for name, meta in case["tensors"].items():
        net.put_tensor(name, st.UniTensor(to_bonds(G.bonds_of(meta)), meta["labels"], G.arr(case["id"], name)))
    r = net.launch()
    ref = G.arr(case["id"], "R")
    assert bonds_meta(r) == case["R"]["bonds"] and r.labels == case["R"]["labels"]
    assert np.linalg.norm(r.elem - ref) <= 1e-13 * max(np.linalg.norm(ref), 1e-300)


def test_fermionic_networks_depend_on_the_gates():
    """Dropping the swap gates changes the result of some fixtures, so the
    fixtures pin the gates."""
    changed = 0
    for case in FNET:
        net = st.Network(text=case["net"])
        for name, meta in case["tensors"].items():
            net.put_tensor(name, st.UniTensor(to_bonds(G.bonds_of(meta)), meta["labels"], G.arr(case["id"], name)))
        net.swaps = [[] for _ in net.tensors]
        r = net.launch()
        changed += not np.allclose(r.elem, G.arr(case["id"], "R"), rtol=1e-12, atol=1e-14)
    assert changed >= 3
