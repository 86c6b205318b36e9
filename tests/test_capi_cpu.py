"""C-ABI checks that need no GPU: the library loads and exports every symbol
the header declares, sector maps equal the oracle's grouping, and every
permute plan -- the kernel's own tile decode and walk, run on the CPU --
moves the elements exactly as the reference does."""
import ctypes as C

import numpy as np
import pytest

from oracle import symtensor as st
from tests import golden_data as G
from trim_gb300 import capi, workloads as wl
from trim_gb300 import uni10 as tu


def to_bonds(spec_bonds):
    return [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in spec_bonds]


def test_exports_every_header_symbol():
    L = capi.lib()
    names = capi.header_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert capi.lib().tn_version() >= 100


def _sectormap_matches(bonds):
    ours = tu.SectorMap(bonds)
    ora = st.grouping(to_bonds(bonds))
    assert ours.elem_num == ora.elem_num
    got = ours.blocks()
    want = [((q.u1, q.prt, q.prtf), r, c, off) for (q, r, c, off) in ora.blocks]
    assert got == want


PERM = [c for c in G.cases().values() if c["kind"] == "permute"]


@pytest.mark.parametrize("case", PERM, ids=[c["id"] for c in PERM])
def test_sectormap_and_permute_plan_match_reference(case):
    bonds = G.bonds_of(case["T"])
    _sectormap_matches(bonds)
    src = tu.SectorMap(bonds)
    # destination bonds as permute builds them (UniTensorReal.cpp:568-580)
    labels, new = case["T"]["labels"], case["new_labels"]
    rsp = [labels.index(l) for l in new]
    out = [wl.change(bonds[rsp[b]], 1 if b < case["rownum"] else -1) for b in range(len(bonds))]
    dst = tu.SectorMap(out)
    x = G.arr(case["id"], "T")
    got, written = tu.plan_check_permute(src, dst, rsp, x)
    assert written == x.size
    assert np.array_equal(got, G.arr(case["id"], "P"))


@pytest.mark.parametrize("case", PERM, ids=[c["id"] for c in PERM])
def test_operand_views_match_reference_permute(case):
    """Where a permute's result is a set of row-major views of its source
    (what the FP64 GEMM reads in place of the permuted copy), the views
    rebuild the reference's permuted elements exactly."""
    bonds = G.bonds_of(case["T"])
    src = tu.SectorMap(bonds)
    labels, new = case["T"]["labels"], case["new_labels"]
    rsp = [labels.index(l) for l in new]
    out = [wl.change(bonds[rsp[b]], 1 if b < case["rownum"] else -1) for b in range(len(bonds))]
    dst = tu.SectorMap(out)
    got = tu.plan_check_views(src, dst, rsp, G.arr(case["id"], "T"))
    if got is not None:
        assert np.array_equal(got, G.arr(case["id"], "P"))


def test_operand_views_cover_the_itebd_regroups():
    """The iTEBD network's regroups (one physical state per charge) are views."""
    spec = wl.itebd()
    A = next(s for s in spec["tensors"] if s.name == "A")
    x = np.arange(wl.elem_count(A.bonds), dtype=np.float64)
    src = tu.SectorMap(A.bonds)
    for rn, rsp in [(1, [0, 1, 2]), (2, [0, 1, 2])]:
        out = [wl.change(A.bonds[rsp[b]], 1 if b < rn else -1) for b in range(3)]
        dst = tu.SectorMap(out)
        want, _ = tu.plan_check_permute(src, dst, rsp, x)
        got = tu.plan_check_views(src, dst, rsp, x)
        if rn == 2:
            assert got is not None and np.array_equal(got, x)  # no move at all
        else:
            assert got is not None and np.array_equal(got, want)


def test_permute_plans_of_workloads_bit_exact():
    rng = np.random.default_rng(7)
    # workload 1's permute, the iTEBD tensors' contract permutes, MERA chi=6
    cases = []
    w1 = wl.u1_rank4()
    cases.append((w1["tensors"][0].bonds, [0, 1, 2, 3], [0, 1, 3, 2], 2))
    it = wl.itebd()
    A = it["tensors"][1]
    cases.append((A.bonds, [10, 1, 11], [1, 11, 10], 1))
    cases.append((A.bonds, [10, 1, 11], [11, 10, 1], 2))
    m = wl.mera(chi=6)
    O = m["tensors"][3]
    cases.append((O.bonds, [0, 1, 2, 3, 4, 5], [4, 5, 0, 1, 2, 3], 2))
    cases.append((O.bonds, [0, 1, 2, 3, 4, 5], [5, 3, 1, 0, 2, 4], 3))
    # the MERA ascend's permutes whose two contiguous bonds are both short:
    # transpose tiles of several stacked planes
    for perm, rn in (((0, 3, 5, 1, 2, 4), 3), ((1, 2, 3, 5, 0, 4), 4), ((2, 3, 5, 0, 1, 4), 3),
                     ((0, 2, 3, 5, 1, 4), 4), ((3, 5, 0, 1, 2, 4), 2)):
        cases.append((O.bonds, [0, 1, 2, 3, 4, 5], list(perm), rn))
    for bonds, labels, new, rn in cases:
        x = rng.uniform(-1, 1, wl.elem_count(bonds))
        t = st.UniTensor(to_bonds(bonds), labels, x)
        t.permute(new, rn)
        rsp = [labels.index(l) for l in new]
        out = [wl.change(bonds[rsp[b]], 1 if b < rn else -1) for b in range(len(bonds))]
        got, written = tu.plan_check_permute(tu.SectorMap(bonds), tu.SectorMap(out), rsp, x)
        assert written == x.size
        assert np.array_equal(got, t.elem)


def test_errors_are_statuses():
    with pytest.raises(capi.TnError) as e:
        tu.SectorMap([(1, [(1, 0, 0, 2)]), (-1, [(0, 0, 0, 2)])])  # no common charge
    assert e.value.code == 8
    with pytest.raises(capi.TnError) as e:
        tu.SectorMap([(-1, [(0, 0, 0, 2)]), (1, [(0, 0, 0, 2)])])  # IN after OUT
    assert e.value.code == 1
    assert "BD_OUT bonds must be placed after all BD_IN bonds" in str(e.value)
    with pytest.raises(capi.TnError):
        tu.SectorMap([(1, [(1000, 0, 0, 2)])])  # U1 out of range
    with pytest.raises(capi.TnError):
        tu.SectorMap([(2, [(0, 0, 0, 2)])])  # bad type


@pytest.mark.parametrize("case", PERM, ids=[c["id"] for c in PERM])
def test_complex_permute_plan_matches_reference(case):
    """The complex (cflag) permute moves 16-byte (re, im) pairs with the
    real permute's sector arithmetic (UniTensorComplex.cpp:592-825 is
    UniTensorReal.cpp:532-768 on Complex elements): with re = T and
    im = -2 T (exact), the result is (P, -2 P) bit for bit, fermionic signs
    on both parts, on tiles of half the real tile limits."""
    bonds = G.bonds_of(case["T"])
    labels, new = case["T"]["labels"], case["new_labels"]
    rsp = [labels.index(l) for l in new]
    out = [wl.change(bonds[rsp[b]], 1 if b < case["rownum"] else -1) for b in range(len(bonds))]
    x = G.arr(case["id"], "T")
    z = x + 1j * (-2.0 * x)
    got, written = tu.plan_check_permute_c128(tu.SectorMap(bonds), tu.SectorMap(out), rsp, z)
    assert written == x.size
    p = G.arr(case["id"], "P")
    assert np.array_equal(got.real, p) and np.array_equal(got.imag, -2.0 * p)


def test_complex_permute_plans_of_dense_tensors():
    """Dense rank-6 complex permutes on all three tile modes (2-D transpose,
    stacked planes of short bonds, long rows) against numpy."""
    rng = np.random.default_rng(8)
    chi = 6
    bonds = [(1, [(0, 0, 0, chi)])] * 3 + [(-1, [(0, 0, 0, chi)])] * 3
    x = rng.uniform(-1, 1, chi ** 6) + 1j * rng.uniform(-1, 1, chi ** 6)
    for perm, rn in (((4, 5, 0, 1, 2, 3), 2), ((0, 3, 5, 1, 2, 4), 3), ((1, 2, 0, 3, 4, 5), 3), ((5, 4, 3, 2, 1, 0), 3)):
        out = [wl.change(bonds[perm[b]], 1 if b < rn else -1) for b in range(6)]
        got, written = tu.plan_check_permute_c128(tu.SectorMap(bonds), tu.SectorMap(out), list(perm), x)
        assert written == x.size
        assert np.array_equal(got, x.reshape([chi] * 6).transpose(perm).reshape(-1))


def test_permute_plan_of_the_ipeps_operand_short_rows():
    """The iPEPS quadrant's big operand permute X[10,3|4,20] -> [3,4|10,20]:
    the combined double-layer bonds carry charge runs of 4, so each
    sub-block row is 4 elements on both sides; the plan stacks them into 3-D
    tiles (mode 3).  Bit-exact against the oracle."""
    rng = np.random.default_rng(9)
    spec = wl.ipeps_ctm(chi=16, D=4)
    _, C, T1, _ = spec["tensors"]
    c_in, dd, c_out = T1.bonds
    bonds = [dd, wl.change(c_in, 1), wl.change(c_out, -1), wl.change(dd, -1)]  # X[10, 3 | 4, 20]
    labels, new, rn = [10, 3, 4, 20], [3, 4, 10, 20], 2
    x = rng.uniform(-1, 1, wl.elem_count(bonds))
    t = st.UniTensor(to_bonds(bonds), labels, x)
    t.permute(new, rn)
    rsp = [labels.index(l) for l in new]
    out = [wl.change(bonds[rsp[b]], 1 if b < rn else -1) for b in range(4)]
    got, written = tu.plan_check_permute(tu.SectorMap(bonds), tu.SectorMap(out), rsp, x)
    assert written == x.size
    assert np.array_equal(got, t.elem)
    z = x + 1j * (0.5 * x)
    gotc, _ = tu.plan_check_permute_c128(tu.SectorMap(bonds), tu.SectorMap(out), rsp, z)
    assert np.array_equal(gotc.real, t.elem) and np.array_equal(gotc.imag, 0.5 * t.elem)
