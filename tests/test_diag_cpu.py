"""The oracle's diagonal contraction (RDotR's diagRowMul / diagColMul applied
to every block, BlockTools.cpp:45-60) against its own dense sector GEMMs on
the same tensors: identical values (a sum with one non-zero term), the
diagonal flag's rules, and the iTEBD network with diagonal Lambdas."""
import numpy as np

from oracle import symtensor as st
from trim_gb300 import workloads as wl


def ob(bonds):
    return [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in bonds]


def diag_tensor(spec, elems):
    t = st.UniTensor(ob(spec.bonds), spec.labels)
    for q, r, c, d in wl.diag_blocks(spec.bonds, elems):
        t.put_block(st.Qnum(*q), d, diag=True, fresh=True)
    return t


def test_diag_flag_rules():
    spec = wl.itebd()
    La = spec["tensors"][0]
    e = wl.gen_elems(La, np.random.default_rng(0))
    t = diag_tensor(La, e)
    assert t.diag and np.array_equal(t.elem, e)
    c = t.copy()
    assert c.diag
    c.permute([10, -1], 1)  # a block-wise transpose keeps it diagonal
    assert c.diag
    q, r, cc, _ = wl.diag_blocks(La.bonds, e)[0]
    t.put_block(st.Qnum(*q), np.ones((r, cc)))
    assert not t.diag


def test_itebd_network_diag_matches_dense():
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    dense, diag = st.Network(text=spec["net"]), st.Network(text=spec["net"])
    for s in spec["tensors"]:
        dense.put_tensor(s.name, st.UniTensor(ob(s.bonds), s.labels, els[s.name]))
        t = diag_tensor(s, els[s.name]) if s.kind == "diag" else st.UniTensor(ob(s.bonds), s.labels, els[s.name])
        diag.put_tensor(s.name, t)
    shapes = []
    got = diag.launch(gemm=lambda a, b: (shapes.append(a.shape + (b.shape[1],)), a @ b)[1]).elem
    want = dense.launch().elem
    assert np.array_equal(got, want)
    assert len(shapes) == 17 + 3  # A.B over 17 charges, the gate over 3; no Lambda GEMM


def test_rectangular_diagonal_rows_beyond_the_diagonal_are_zero():
    # Lambda[x | y] with x of dim 5 and y of dim 3 in one charge: a 5 x 3 block
    bx = st.Bond.from_runs(st.BD_IN, [(st.Qnum(0), 5)])
    by = st.Bond.from_runs(st.BD_OUT, [(st.Qnum(0), 3)])
    lam = st.UniTensor([bx, by], labels=[1, 2])
    lam.put_block(st.Qnum(0), np.array([2.0, -3.0, 0.5]), diag=True, fresh=True)
    assert lam.diag
    rng = np.random.default_rng(1)
    x = st.UniTensor([by.copy().change(st.BD_IN), st.Bond.from_runs(st.BD_OUT, [(st.Qnum(0), 4)])], labels=[2, 3],
                     elem=rng.standard_normal(12))
    dense = st.UniTensor([bx, by], labels=[1, 2], elem=lam.elem)
    got = st.contract(lam, x).elem.reshape(5, 4)
    want = st.contract(dense, x).elem.reshape(5, 4)
    assert np.array_equal(got, want)
    assert np.all(got[3:] == 0.0)
