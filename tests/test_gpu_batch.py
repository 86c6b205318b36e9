"""Batches of independent contractions (uni10::Batch, tn_batch_*): one
grouped launch over a work list planned once, a CUDA graph of it, and the
per-sector loop baseline (tn_contract_sectors_loop).  Every output is what
contract(a[i], b[i]) gives (the oracle within 1e-13; split precision within
1e-12 of FP64), replays are bit-identical to the eager launch, and new
elements put into the batch are picked up by the replay."""
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


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_pairs(tu, n, seed, hi=96, permuted_b=False):
    spec = wl.batched(n=n, hi=hi, seed=seed)
    rng = np.random.default_rng(spec["seed"])
    A, B, OA, OB = [], [], [], []
    for t1, t2 in spec["pairs"]:
        e1, e2 = wl.gen_elems(t1, rng), wl.gen_elems(t2, rng)
        a, b = tu.UniTensor(t1.bonds, t1.labels, e1), tu.UniTensor(t2.bonds, t2.labels, e2)
        oa, obt = st.UniTensor(ob(t1.bonds), t1.labels, e1), st.UniTensor(ob(t2.bonds), t2.labels, e2)
        if permuted_b:  # B stored as (w | y, z): the batch permutes it back to (y, z | w)
            b.permute([3, 1, 2], 1)
            obt.permute([3, 1, 2], 1)
        A.append(a)
        B.append(b)
        OA.append(oa)
        OB.append(obt)
    return A, B, OA, OB


@pytest.mark.parametrize("permuted_b", [False, True])
def test_batch_launch_capture_replay(tu, permuted_b):
    A, B, OA, OB = make_pairs(tu, 40, 11, permuted_b=permuted_b)
    bt = tu.Batch(A, B)
    bt.launch("fp64")
    eager = [bt.output(i).get_elem() for i in range(len(A))]
    want = [st.contract(a, b).elem for a, b in zip(OA, OB)]
    assert max(rel(g, w) for g, w in zip(eager, want)) <= 1e-13
    bt.capture("fp64")
    bt.replay()
    tu.sync()
    assert all(np.array_equal(bt.output(i).get_elem(), e) for i, e in enumerate(eager))
    # new elements for two pairs, then a replay
    for i in (0, 39):  # the same bonds with new values
        a = A[i].copy()
        b = B[i].copy()
        a.set_elem(np.random.default_rng(100 + i).uniform(-1, 1, a.elem_num()))
        b.set_elem(np.random.default_rng(200 + i).uniform(-1, 1, b.elem_num()))
        bt.put(i, a, b)
        OA[i] = st.UniTensor(OA[i].bonds, OA[i].labels, a.get_elem())
        OB[i] = st.UniTensor(OB[i].bonds, OB[i].labels, b.get_elem())
    bt.replay()
    tu.sync()
    for i in (0, 1, 39):
        assert rel(bt.output(i).get_elem(), st.contract(OA[i], OB[i]).elem) <= 1e-13


def test_batch_split_and_per_sector_loop(tu):
    A, B, OA, OB = make_pairs(tu, 32, 13, hi=128)
    bt = tu.Batch(A, B)
    bt.launch("fp64")
    f64 = [bt.output(i).get_elem() for i in range(len(A))]
    bt.launch("split")
    spl = [bt.output(i).get_elem() for i in range(len(A))]
    assert max(rel(s, f) for s, f in zip(spl, f64)) <= 1e-12
    secs = bt.sectors()
    assert len(secs) > len(A)
    tu.contract_sectors_loop("fp64", secs, 0, 0, 0)  # absolute addresses: one launch per sector
    tu.sync()
    loop = [bt.output(i).get_elem() for i in range(len(A))]
    assert max(rel(l, f) for l, f in zip(loop, f64)) <= 1e-13


def test_batch_refuses_outer_products(tu):
    from trim_gb300.capi import TnError

    a = tu.UniTensor([wl.dense_bond(1, 3), wl.dense_bond(-1, 4)], [1, 2], np.ones(12))
    b = tu.UniTensor([wl.dense_bond(1, 2), wl.dense_bond(-1, 2)], [3, 4], np.ones(4))
    with pytest.raises(TnError):
        tu.Batch([a], [b])
