"""Checks shared by the CPU and GPU tests of Block::eigh.

An eigendecomposition is compared by what is unique about it: the
eigenvalues (ascending), and for every cluster of equal eigenvalues the
orthogonal projector onto its eigenvectors (eigenvector signs and the basis
inside a repeated eigenvalue's space are arbitrary, in dsyev as here)."""
import numpy as np

from oracle import symtensor as st
from tests import golden_data as G


def sym_lower(a):
    """The matrix dsyev 'U' sees in the reference's row-major buffer."""
    a = np.asarray(a, dtype=np.float64)
    return np.tril(a) + np.tril(a, -1).T


def golden_eigh_blocks(case_id):
    """[(block, E_ref, V_ref)] of a golden eigh case, in Qnum order."""
    c = G.cases()[case_id]
    bonds = [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in G.bonds_of(c)]
    t = st.UniTensor(bonds, [1, 2], G.arr(case_id, "elem"))
    out = []
    for j, q in enumerate(t.block_qnums()):
        out.append((t.get_block(q), G.arr(case_id, f"E{j}"), G.arr(case_id, f"V{j}")))
    return out


def clusters(e, gap):
    """Index ranges of eigenvalues closer than gap to their neighbour."""
    out, start = [], 0
    for i in range(1, len(e) + 1):
        if i == len(e) or e[i] - e[i - 1] > gap:
            out.append((start, i))
            start = i
    return out


def check_eigh(a, e, v, e_ref, v_ref=None, tol=1e-13, dk=1e-12):
    """e ascending and within tol * max|e_ref| of e_ref; V orthonormal rows,
    V^T diag(e) V = sym(a) within 10 tol ||sym(a)||_F; the projector of every
    eigenvalue cluster equal to the reference's within the Davis-Kahan bound
    dk * max|e_ref| / gap (gap: distance to the nearest eigenvalue outside
    the cluster; eigenvectors of both sides carry errors of that size)."""
    s = sym_lower(a)
    n = s.shape[0]
    e, v = np.asarray(e).ravel(), np.asarray(v).reshape(n, n)
    scale = max(float(np.max(np.abs(e_ref))) if n else 0.0, 1e-300)
    assert np.all(np.diff(e) >= 0), "eigenvalues not ascending"
    assert np.max(np.abs(e - e_ref), initial=0.0) <= tol * scale
    assert np.max(np.abs(v @ v.T - np.eye(n)), initial=0.0) <= tol * 10
    ns = max(np.linalg.norm(s), 1e-300)
    assert np.linalg.norm(v.T @ np.diag(e) @ v - s) <= tol * 10 * ns
    if v_ref is not None:
        v_ref = np.asarray(v_ref).reshape(n, n)
        er = np.asarray(e_ref)
        for lo, hi in clusters(er, 1e-8 * scale):
            if hi - lo == n:
                continue  # one cluster: the projector is the identity
            gap = min(er[lo] - er[lo - 1] if lo > 0 else np.inf, er[hi] - er[hi - 1] if hi < n else np.inf)
            p = v[lo:hi].T @ v[lo:hi]
            pr = v_ref[lo:hi].T @ v_ref[lo:hi]
            assert np.max(np.abs(p - pr)) <= max(dk * scale / gap, dk), f"eigenvectors {lo}:{hi} differ"
