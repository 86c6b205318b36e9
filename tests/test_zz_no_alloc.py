"""The fixed-scratch FP64 sector-GEMM entry point, for callers that cannot
allocate device memory (a framework that owns all of the GPU's memory through
its own allocator, a latency-critical loop, a plugin host that forbids
allocation after start-up).  Through the C ABI it must give the same result
as the regular entry point, tn_contract_sectors, within the FP64 tolerance of
the other tests, on two calls in a row that reuse the shared scratch array,
and it must reject work larger than that array.

This file is collected last on purpose; it also passes on its own in a fresh
process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-13


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from trim_gb300 import capi
    from trim_gb300 import uni10 as tu

    stream = torch.cuda.current_stream()
    tu.set_stream(stream.cuda_stream)  # both entry points on one stream
    return torch, capi, stream


def _sectors(shapes):
    """Packed row-major A, B, C layouts for a list of (M, N, K)."""
    out, ao, bo, co = [], 0, 0, 0
    for m, n, k in shapes:
        out.append((m, n, k, ao, bo, co))
        ao += m * k
        bo += k * n
        co += m * n
    return out, ao, bo, co


def _run(env, shapes, seed):
    torch, capi, stream = env
    gemms, na, nb, nc = _sectors(shapes)
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.rand(na, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    B = torch.rand(nb, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    ref = torch.zeros(nc, dtype=torch.float64, device="cuda")
    got = torch.full((nc,), float("nan"), dtype=torch.float64, device="cuda")
    arr = (capi.SectorGemm * len(gemms))(*[capi.SectorGemm(*x) for x in gemms])
    capi.call("tn_contract_sectors", None, capi.MODE_FP64, len(gemms), arr, A.data_ptr(), B.data_ptr(), ref.data_ptr())
    capi.call("tn_contract_sectors_fp64_noalloc", C.c_void_p(stream.cuda_stream), len(gemms), arr, A.data_ptr(),
              B.data_ptr(), got.data_ptr())
    torch.cuda.synchronize()
    r, o = ref.cpu().numpy(), got.cpu().numpy()
    return float(np.linalg.norm(o - r) / np.linalg.norm(r)), o, (A.cpu().numpy(), B.cpu().numpy(), gemms)


def test_noalloc_matches_regular_entry_point_twice(env):
    # call 1: mixed sector sizes, few tiles -> K is split (partials in the scratch)
    e1, out1, (a, b, gemms) = _run(env, [(130, 128, 68), (2, 3, 5), (64, 64, 600), (1, 1, 1), (33, 17, 9)], 11)
    assert e1 <= FP64_TOL
    # the result is also the product itself (one sector checked on the host)
    m, n, k, ao, bo, co = gemms[2]
    want = a[ao:ao + m * k].reshape(m, k) @ b[bo:bo + k * n].reshape(k, n)
    assert np.linalg.norm(out1[co:co + m * n].reshape(m, n) - want) <= FP64_TOL * np.linalg.norm(want)
    # call 2, right after: other shapes and split counts; stale scratch
    # contents from call 1 must not leak into the result
    e2, _, _ = _run(env, [(300, 257, 40), (17, 520, 3), (96, 96, 96)], 12)
    assert e2 <= FP64_TOL


def test_noalloc_rejects_work_beyond_the_fixed_scratch(env):
    torch, capi, stream = env
    A = torch.zeros(16, dtype=torch.float64, device="cuda")
    big = (capi.SectorGemm * 1)(capi.SectorGemm(4096, 4096, 1, 0, 0, 0))  # 32768 tiles of 16x32
    with pytest.raises(capi.TnError) as e:
        capi.call("tn_contract_sectors_fp64_noalloc", C.c_void_p(stream.cuda_stream), 1, big, A.data_ptr(),
                  A.data_ptr(), A.data_ptr())
    assert e.value.code == 1  # TN_ERR_ARG
    assert "fixed scratch" in str(e.value)


def test_noalloc_narrow_sectors_and_many_items(env):
    # sectors with N <= 8 and 32 <= K take 16-row items (lanes along K); more
    # items than 16 per SM makes the planner order them by cost
    torch, capi, stream = env
    shapes = [(200, 5, 64), (64, 3, 40), (37, 8, 33)] + [(8, 8, 8)] * 3000
    for seed in (21, 22):  # two calls in a row over the shared array
        err, out, (a, b, gemms) = _run(env, shapes, seed)
        assert err <= FP64_TOL
        for m, n, k, ao, bo, co in gemms[:3] + gemms[-2:]:
            want = a[ao:ao + m * k].reshape(m, k) @ b[bo:bo + k * n].reshape(k, n)
            assert np.linalg.norm(out[co:co + m * n].reshape(m, n) - want) <= FP64_TOL * np.linalg.norm(want)


def test_noalloc_drops_the_k_split_near_the_item_limit(env):
    # 11 800 one-tile sectors plus one long-K sector: the K-split plan needs
    # more work items than the fixed list holds (11 915), the unsplit plan fits
    _, _, stream = env
    shapes = [(1, 1, 1)] * 11800 + [(16, 32, 200000)]
    err, out, (a, b, gemms) = _run(env, shapes, 31)
    assert err <= FP64_TOL
    m, n, k, ao, bo, co = gemms[-1]
    want = a[ao:ao + m * k].reshape(m, k) @ b[bo:bo + k * n].reshape(k, n)
    assert np.linalg.norm(out[co:co + m * n].reshape(m, n) - want) <= FP64_TOL * np.linalg.norm(want)


def test_noalloc_refuses_a_capturing_stream(env):
    # the work list comes from host memory that dies with the call, so a call
    # on a stream under capture is refused before it issues anything, and the
    # caller's capture is left usable
    torch, capi, _ = env
    gemms, na, nb, nc = _sectors([(64, 64, 64)])
    A = torch.ones(na, dtype=torch.float64, device="cuda")
    x = torch.arange(16, dtype=torch.float64, device="cuda")
    y = torch.zeros(16, dtype=torch.float64, device="cuda")
    arr = (capi.SectorGemm * 1)(capi.SectorGemm(*gemms[0]))
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    code = None
    with torch.cuda.graph(g):
        y.copy_(x * 2)
        try:
            capi.call("tn_contract_sectors_fp64_noalloc", C.c_void_p(torch.cuda.current_stream().cuda_stream), 1, arr,
                      A.data_ptr(), A.data_ptr(), A.data_ptr())
        except capi.TnError as e:
            code = e.code
    assert code == 7  # TN_ERR_UNSUPPORTED
    x += 1
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(y, (x * 2))
