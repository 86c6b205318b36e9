"""GPU parity of the per-sector FP64 SVD (Block::svd) and of the iTEBD
truncation, through the C ABI, against LAPACK (the oracle) and the reference's
golden singular values of the iTEBD theta.

Tolerances: singular values within 1e-13 of the largest one of their sector;
||U S VT - A||_F <= 1e-13 ||A||_F; ||U^T U - I||_max and ||VT VT^T - I||_max
<= 1e-13 (columns of nonzero singular values); truncation: kept counts
identical, norm within 1e-13, reconstruction of the kept part within 1e-12."""
import numpy as np
import pytest

from oracle import symtensor as st
from tests import golden_data as G

pytestmark = pytest.mark.gpu

TOL = 1e-13


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from trim_gb300 import capi
    from trim_gb300 import uni10 as tu

    tu.set_stream(torch.cuda.current_stream().cuda_stream)
    return torch, capi, tu


def run_svd(env, mats):
    """All matrices in one batched call; returns [(U, S, VT)], sweeps."""
    torch, capi, tu = env
    secs, ao, uo, so, vo = [], 0, 0, 0, 0
    for a in mats:
        M, N = a.shape
        k = min(M, N)
        secs.append((M, N, ao, uo, so, vo))
        ao += M * N
        uo += M * k
        so += k
        vo += k * N
    A = torch.from_numpy(np.concatenate([a.ravel() for a in mats])).cuda()
    U = torch.full((max(uo, 1),), np.nan, dtype=torch.float64, device="cuda")
    S = torch.full((max(so, 1),), np.nan, dtype=torch.float64, device="cuda")
    VT = torch.full((max(vo, 1),), np.nan, dtype=torch.float64, device="cuda")
    sweeps = tu.svd_sectors(secs, A.data_ptr(), U.data_ptr(), S.data_ptr(), VT.data_ptr(), sweeps=True)
    tu.sync()
    u, s, vt = U.cpu().numpy(), S.cpu().numpy(), VT.cpu().numpy()
    out = []
    for (M, N, _, uo, so, vo) in secs:
        k = min(M, N)
        out.append((u[uo:uo + M * k].reshape(M, k), s[so:so + k], vt[vo:vo + k * N].reshape(k, N)))
    return out, sweeps


def check_svd(a, u, s, vt, tol=TOL):
    ref = np.linalg.svd(a, compute_uv=False)
    smax = max(ref.max(), 1e-300)
    assert np.all(np.diff(s) <= 0), "singular values not descending"
    assert np.max(np.abs(s - ref)) <= tol * smax
    na = max(np.linalg.norm(a), 1e-300)
    assert np.linalg.norm(u @ np.diag(s) @ vt - a) <= tol * na
    nz = s > 1e-300
    k = int(nz.sum())
    uu, vv = u[:, nz], vt[nz, :]
    assert np.max(np.abs(uu.T @ uu - np.eye(k))) <= tol
    assert np.max(np.abs(vv @ vv.T - np.eye(k))) <= tol


SHAPES = [(1, 1), (1, 7), (7, 1), (2, 2), (5, 3), (3, 5), (16, 16), (33, 17), (17, 33), (64, 64), (37, 37),
          (83, 83), (106, 106), (130, 130), (200, 40), (40, 200), (256, 256), (300, 300)]


def test_svd_batched_shapes(env):
    rng = np.random.default_rng(11)
    mats = [rng.uniform(-1, 1, size=s) for s in SHAPES]
    res, sweeps = run_svd(env, mats)
    for a, (u, s, vt), sw, shp in zip(mats, res, sweeps, SHAPES):
        assert 0 < sw % 100 < 40 and sw // 100 <= 2 * 20, (shp, sw)  # two FP32 passes
        check_svd(a, u, s, vt)


def test_svd_cusolver_fallback_and_empty(env):
    rng = np.random.default_rng(12)
    mats = [rng.standard_normal((600, 600)), rng.standard_normal((1, 1))]
    res, sweeps = run_svd(env, mats)
    assert sweeps[0] == 0  # too large for the cluster kernel: cuSOLVER
    check_svd(mats[0], *res[0], tol=1e-12)
    check_svd(mats[1], *res[1])


def test_svd_graded_and_rank_deficient(env):
    rng = np.random.default_rng(13)
    q1, _ = np.linalg.qr(rng.standard_normal((50, 50)))
    q2, _ = np.linalg.qr(rng.standard_normal((50, 50)))
    graded = q1 @ np.diag(np.logspace(0, -12, 50)) @ q2.T
    rank3 = rng.standard_normal((40, 3)) @ rng.standard_normal((3, 30))
    zero_col = rng.standard_normal((20, 10))
    zero_col[:, 4] = 0.0
    # sectors of >= 16 columns start from the QR preconditioner, whose V
    # completion replaces the columns of numerically zero singular values
    rank1 = np.outer(rng.standard_normal(60), rng.standard_normal(48))
    zero = np.zeros((40, 40))
    mats = [graded, rank3, zero_col, rank1, zero]
    res, _ = run_svd(env, mats)
    for a, (u, s, vt) in zip(mats[3:], res[3:]):
        ref = np.linalg.svd(a, compute_uv=False)
        assert np.max(np.abs(s - ref)) <= TOL * max(ref.max(), 1e-300)
        assert np.linalg.norm(u @ np.diag(s) @ vt - a) <= TOL * max(np.linalg.norm(a), 1e-300)
    assert not np.any(res[4][1])  # the zero sector: zero singular values
    check_svd(graded, *res[0])
    u, s, vt = res[1]
    ref = np.linalg.svd(rank3, compute_uv=False)
    assert np.max(np.abs(s - ref)) <= TOL * ref.max()
    assert np.linalg.norm(u @ np.diag(s) @ vt - rank3) <= TOL * np.linalg.norm(rank3)
    u, s, vt = res[2]
    assert np.linalg.norm(u @ np.diag(s) @ vt - zero_col) <= TOL * np.linalg.norm(zero_col)


def golden_theta():
    meta = G.cases()["itebd"]["TH"]
    bonds = [st.Bond.from_runs(t, [(st.Qnum(u, p, f), d) for (u, p, f, d) in runs]) for t, runs in G.bonds_of(meta)]
    return st.UniTensor(bonds, meta["labels"], G.arr("itebd", "TH")), meta


def test_itebd_theta_singular_values_match_reference(env):
    th, _ = golden_theta()
    blocks = [th.get_block(q) for q in th.block_qnums()]
    res, sweeps = run_svd(env, blocks)
    sref = G.arr("itebd", "S")  # the compiled reference's dgesvd, per block in Qnum order
    s = np.concatenate([r[1] for r in res])
    assert np.max(np.abs(s - sref)) <= TOL * sref.max()
    for b, (u, sv, vt) in zip(blocks, res):
        check_svd(b, u, sv, vt)
    assert all(0 < sw % 100 < 40 for sw in sweeps)


def test_truncate_sectors_ties_and_limits(env):
    torch, capi, tu = env
    vals = [np.array([3.0, 2.0, 1.0]), np.array([3.0, 2.0, 1.0]), np.array([2.5])]
    for chi in (1, 2, 3, 4, 5, 7, 100):
        S = torch.from_numpy(np.concatenate(vals)).cuda()
        kept, norm = tu.truncate_sectors([0, 3, 6], [3, 3, 1], S.data_ptr(), chi)
        k_ref, n_ref, s_ref = st.truncate_global(vals, chi)
        assert kept == k_ref, chi
        assert abs(norm - n_ref) <= TOL * n_ref
        got = S.cpu().numpy()
        for q, (o, k) in enumerate(zip([0, 3, 6], kept)):
            assert np.allclose(got[o:o + k], s_ref[q], rtol=1e-15, atol=0)


def test_itebd_svd_truncate_matches_oracle(env):
    torch, capi, tu = env
    th, meta = golden_theta()
    t = tu.UniTensor(G.bonds_of(meta), meta["labels"], G.arr("itebd", "TH"))
    U, S, VT, norm = t.svd_truncate(512)
    Uo, So, VTo, norm_o = st.svd_truncate(th, 512)
    assert abs(norm - norm_o) <= TOL * norm_o
    assert [list(map(list, r)) for _, r in S.bonds()] == [[[q.u1, q.prt, q.prtf, d] for q, d in zip(b.qnums, b.qdegs)]
                                                           for b in So.bonds]
    assert np.max(np.abs(S.get_elem() - So.elem)) <= TOL
    # U S VT rebuilds the rank-512 part of theta like the oracle's factors
    rec = tu.contract(tu.contract(U, S), VT)
    rec.permute(meta["labels"], th.in_bond_num())
    rec_o = st.contract(st.contract(Uo, So), VTo).permute(th.labels, th.in_bond_num())
    assert np.linalg.norm(rec.get_elem() - rec_o.elem) <= 1e-12 * np.linalg.norm(rec_o.elem)
