"""SVD and truncation checks that need no GPU.

* The cluster shapes the library plans for every sector of the workloads fit
  the shared memory of a CTA.
* The Jacobi kernel's tournament (the index arithmetic of
  trim_gb300/csrc/kernels/svd_jacobi.cu, restated here) visits every column
  pair exactly once per sweep, never gives one column to two warps in the
  same sub-round, and its block exchange is a permutation of the slots.
* The oracle's global truncation follows its stated order and normalises.
* The QR preconditioner of the first FP32 pass, restated in numpy FP32,
  gives a nonsingular start that two Newton-Schulz steps make orthogonal in
  FP64, on random, graded, rank-deficient and zero blocks.
"""
import itertools

import numpy as np
import pytest

from oracle import symtensor as st
from tests import golden_data as G
from trim_gb300 import uni10 as tu

SMEM_LIMIT = 227 * 1024
ITEBD_SECTORS = [2, 5, 11, 22, 37, 58, 83, 106, 123, 130, 123, 106, 83, 58, 37, 22, 11, 5, 2]


def test_plan_fits_shared_memory():
    shapes = [(n, n) for n in ITEBD_SECTORS] + [(1, 1), (1, 9), (9, 1), (200, 40), (40, 200), (300, 300),
                                                 (256, 256), (24, 576), (1000, 3)]
    for M, N in shapes:
        p = tu.svd_plan(M, N)
        assert p["P"] in (1, 2, 4, 8, 16), (M, N, p)
        assert p["smem"] <= SMEM_LIMIT
        nx = min(M, N)
        assert 2 * p["P"] * p["b"] >= nx
        assert p["L"] % 2 == 0 and p["L"] >= M + N
        if p["P"] < 16:
            assert p["b"] <= 8
    # too large for shared memory: the cuSOLVER fallback
    assert tu.svd_plan(600, 600)["P"] == 0
    assert tu.svd_plan(20000, 4)["P"] == 0
    # a device that schedules clusters of at most 8
    p = tu.svd_plan(130, 130, max_cluster=8)
    assert p["P"] == 8 and p["b"] == 9


def _tournament(P, b, nx):
    """The kernel's schedule: per sweep, the list of sub-rounds, each a list
    of (cta, column i, column j) in global column ids."""
    nblk = 2 * P
    pos_blk = list(range(nblk))  # round-0 layout: position k holds block k
    subrounds = []
    for rnd in range(nblk - 1):
        holders = {}  # cta -> (slot0 block, slot1 block)
        for cta in range(P):
            holders[cta] = (pos_blk[cta], pos_blk[nblk - 1 - cta])
        if rnd == 0:
            bb = b + (b & 1)
            half = bb // 2
            for s in range(bb - 1):
                sr = []
                for cta in range(P):
                    for p in range(bb):
                        slot, k = divmod(p, half)
                        if k == 0:
                            i, j = s, bb - 1
                        else:
                            i, j = (s + k) % (bb - 1), (s - k + bb - 1) % (bb - 1)
                        if i < b and j < b:
                            blk = holders[cta][slot]
                            sr.append((cta, blk * b + i, blk * b + j))
                subrounds.append(sr)
        for s in range(b):
            sr = []
            for cta in range(P):
                b0, b1 = holders[cta]
                for i in range(b):
                    sr.append((cta, b0 * b + i, b1 * b + (i + s) % b))
            subrounds.append(sr)
        if P > 1:
            # exchange: position k -> k+1, 2P-1 -> 1, 0 stays; check the
            # destination slots form a permutation
            dest = []
            for cta in range(P):
                for slot in range(2):
                    pos = cta if slot == 0 else nblk - 1 - cta
                    npos = 0 if pos == 0 else (1 if pos == nblk - 1 else pos + 1)
                    dcta = npos if npos < P else nblk - 1 - npos
                    dslot = 0 if npos < P else 1
                    assert 0 <= dcta < P
                    dest.append((dcta, dslot, pos_blk[pos], npos))
            assert len({(d[0], d[1]) for d in dest}) == 2 * P
            new = [None] * nblk
            for _, _, blk, npos in dest:
                new[npos] = blk
            pos_blk = new
    assert pos_blk == list(range(nblk))  # a sweep returns to the round-0 layout
    return subrounds


@pytest.mark.parametrize("P,b", [(1, 1), (1, 2), (1, 3), (1, 8), (2, 5), (2, 6), (4, 5), (4, 8), (8, 7),
                                 (8, 8), (16, 5), (16, 9), (4, 17), (8, 19), (2, 24), (1, 23)])
def test_tournament_visits_every_pair_once(P, b):
    nx = 2 * P * b
    seen = {}
    for sr in _tournament(P, b, nx):
        used = set()
        for cta, i, j in sr:
            assert i != j
            for c in (i, j):
                assert c not in used  # one warp per column in a sub-round
                used.add(c)
            key = (min(i, j), max(i, j))
            seen[key] = seen.get(key, 0) + 1
    want = {(i, j) for i, j in itertools.combinations(range(nx), 2)}
    assert set(seen) == want
    assert all(v == 1 for v in seen.values())


def test_tournament_of_planned_itebd_sectors():
    for n in sorted(set(ITEBD_SECTORS)):
        p = tu.svd_plan(n, n)
        subs = _tournament(p["P"], p["b"], n)
        pairs = {(min(i, j), max(i, j)) for sr in subs for _, i, j in sr if i < n and j < n}
        assert len(pairs) == n * (n - 1) // 2


def test_truncate_global_order_and_norm():
    s = [np.array([3.0, 2.0, 1.0]), np.array([3.0, 2.0, 1.0]), np.array([2.5])]
    assert st.truncate_global(s, 1)[0] == [1, 0, 0]  # ties go to the lower sector first
    assert st.truncate_global(s, 2)[0] == [1, 1, 0]
    kept, norm, sn = st.truncate_global(s, 3)
    assert kept == [1, 1, 1]
    assert norm == pytest.approx(np.sqrt(9 + 9 + 6.25))
    assert np.allclose(np.concatenate(sn), np.array([3, 3, 2.5]) / norm)
    assert st.truncate_global(s, 4)[0] == [2, 1, 1]
    assert st.truncate_global(s, 5)[0] == [2, 2, 1]
    assert st.truncate_global(s, 100)[0] == [3, 3, 1]


def golden_theta():
    meta = G.cases()["itebd"]["TH"]
    bonds = [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in G.bonds_of(meta)]
    return st.UniTensor(bonds, meta["labels"], G.arr("itebd", "TH"))


def test_itebd_svd_truncate_oracle():
    """The oracle's truncated factors rebuild the rank-chi part of theta."""
    th = golden_theta()
    U, S, VT, norm = st.svd_truncate(th, 512)
    assert U.bonds[-1].dim() == 512 and S.elem_num() == sum(d * d for d in U.bonds[-1].qdegs)
    gold = np.sort(G.arr("itebd", "S"))[::-1]
    assert norm == pytest.approx(np.linalg.norm(gold[:512]), rel=1e-12)
    rec = st.contract(st.contract(U, S), VT)
    rec = rec.permute(th.labels, th.in_bond_num())
    # theta minus its rank-512 part: the discarded singular values
    err = np.linalg.norm(rec.elem * norm - th.elem)
    assert err == pytest.approx(np.linalg.norm(gold[512:]), rel=1e-9)


# ---- the QR preconditioner of the first FP32 pass (svd_qr_kernel,
# svd_v1_kernel in trim_gb300/csrc/kernels/svd_jacobi.cu), restated in numpy
# FP32: columns sorted by decreasing norm, unpivoted Householder QR, one-sided
# Jacobi on R^T, V = P W with the columns normalised and the numerically zero
# ones completed by the unit vector of least row norm, orthogonalised twice.
# The Newton-Schulz steps that follow need V nonsingular and near orthogonal.

def _house_r32(x):
    x = x.astype(np.float32).copy()
    m, n = x.shape
    for k in range(n):
        s2 = np.float32(np.dot(x[k:, k], x[k:, k]))
        x0 = x[k, k]
        nx = np.float32(np.sqrt(s2))
        alpha = -nx if x0 >= 0 else nx
        v0 = np.float32(x0 - alpha)
        vv = np.float32(v0 * v0 + (s2 - x0 * x0))
        if vv <= 0:
            continue
        v = x[k:, k].copy()
        v[0] = v0
        for c in range(k + 1, n):
            f = np.float32(2 * np.dot(v, x[k:, c]) / vv)
            x[k:, c] -= f * v
        x[k, k] = alpha
    return np.triu(x[:n, :n])


def _jacobi32(y, tol=1e-5, sweeps=30):
    """One-sided Jacobi on the columns of y (FP32), cyclic order."""
    y = y.astype(np.float32).copy()
    n = y.shape[1]
    for _ in range(sweeps):
        rot = 0
        for i in range(n - 1):
            for j in range(i + 1, n):
                a, b = np.dot(y[:, i], y[:, i]), np.dot(y[:, j], y[:, j])
                g = np.dot(y[:, i], y[:, j])
                if a <= 0 or b <= 0 or g * g <= tol * tol * a * b:
                    continue
                rot += 1
                z = (b - a) / (2 * g)
                t = np.sign(z) / (abs(z) + np.sqrt(1 + z * z)) if z != 0 else 1.0
                c = 1 / np.sqrt(1 + t * t)
                s = c * t
                yi, yj = y[:, i].copy(), y[:, j].copy()
                y[:, i], y[:, j] = c * yi - s * yj, s * yi + c * yj
        if rot == 0:
            break
    return y


def _precond_v(x):
    n = x.shape[1]
    p = np.argsort(-np.linalg.norm(x, axis=0), kind="stable")
    w = _jacobi32(_house_r32(x[:, p]).T)      # Y V_y, Y = R^T
    v = np.zeros((n, n))
    v[p, :] = w
    cn = np.sum(v * v, axis=0)
    good = cn > 1e-12 * cn.max() if cn.max() > 0 else np.zeros(n, bool)
    v[:, good] /= np.sqrt(cn[good])
    v[:, ~good] = 0
    vs = v.astype(np.float32)
    for g in np.nonzero(~good)[0]:
        k = int(np.argmin(np.sum(vs * vs, axis=1)))  # least row norm: e_k most outside the span
        u = np.zeros(n, np.float32)
        u[k] = 1
        for _ in range(2):
            u -= vs @ (vs.T @ u)
        vs[:, g] = u / np.linalg.norm(u)
        v[:, g] = vs[:, g]
    return v


def _ns2(q):
    for _ in range(2):
        g = q.T @ q
        q = q @ (1.5 * np.eye(len(g)) - 0.25 * (g + g.T))
    return q


@pytest.mark.parametrize("kind", ["random", "graded", "rank2", "zero_col", "zero"])
def test_qr_preconditioner_start_is_orthogonal(kind):
    rng = np.random.default_rng(21)
    m, n = 24, 18
    if kind == "random":
        x = rng.standard_normal((m, n))
    elif kind == "graded":
        x = rng.standard_normal((m, n)) * np.logspace(0, -9, n)
    elif kind == "rank2":
        x = rng.standard_normal((m, 2)) @ rng.standard_normal((2, n))
    elif kind == "zero_col":
        x = rng.standard_normal((m, n))
        x[:, 5] = 0
    else:
        x = np.zeros((m, n))
    q1 = _ns2(_precond_v(x))
    assert np.max(np.abs(q1.T @ q1 - np.eye(n))) < 1e-13  # a valid start for the FP64 stages
    # X Q1: the columns of the leading singular values (above 1e-2 of the
    # largest) are orthogonal to FP32 accuracy; the small ones are left to the
    # second FP32 pass and the FP64 sweeps, as without the preconditioner
    x1 = x @ q1
    gm = x1.T @ x1
    d = np.sqrt(np.diag(gm))
    big = d > 1e-2 * max(d.max(), 1e-300)
    if big.sum() > 1:
        off = np.abs(gm[np.ix_(big, big)]) / np.outer(d[big], d[big])
        np.fill_diagonal(off, 0)
        assert off.max() < 1e-3
