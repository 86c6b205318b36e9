"""Tensor-core sector GEMMs (tcgen05): split precision must stay within
1e-12 relative Frobenius error of FP64 on every workload; the fast BF16 mode
is reported with its (BF16-level) error."""
import numpy as np
import pytest

from tests import golden_data as G
from trim_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

SPLIT_TOL = 1e-12


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from trim_gb300 import capi
    from trim_gb300 import uni10 as tu

    tu.set_stream(torch.cuda.current_stream().cuda_stream)
    return torch, capi, tu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _sectors(shapes):
    out, ao, bo, co = [], 0, 0, 0
    for m, n, k in shapes:
        out.append((m, n, k, ao, bo, co))
        ao += m * k
        bo += k * n
        co += m * n
    return out, ao, bo, co


def _grouped(env, mode, shapes, seed, dist="uniform"):
    torch, capi, tu = env
    gemms, na, nb, nc = _sectors(shapes)
    rng = np.random.default_rng(seed)
    if dist == "uniform":
        a, b = rng.uniform(-1, 1, na), rng.uniform(-1, 1, nb)
    else:
        a, b = rng.standard_normal(na), rng.standard_normal(nb)
    A = torch.from_numpy(a).cuda()
    B = torch.from_numpy(b).cuda()
    Cd = torch.zeros(nc, dtype=torch.float64, device="cuda")
    tu.contract_sectors(mode, gemms, A.data_ptr(), B.data_ptr(), Cd.data_ptr())
    tu.sync()
    c = Cd.cpu().numpy()
    errs = []
    for m, n, k, ao, bo, co in gemms:
        want = a[ao:ao + m * k].reshape(m, k) @ b[bo:bo + k * n].reshape(k, n)
        errs.append(rel(c[co:co + m * n].reshape(m, n), want))
    return errs


# the tensor-core forms: chosen by size, fused (one launch, per-item slicing)
# and tiled (maxima + slices once, pipelined GEMM)
SPLIT_FORMS = ("split_tc", "split_fused", "split_tiled")


@pytest.mark.parametrize("mode", SPLIT_FORMS)
def test_split_single_tile(env, mode):
    errs = _grouped(env, mode, [(128, 64, 64)], 1)
    assert errs[0] <= SPLIT_TOL, errs


@pytest.mark.parametrize("mode", SPLIT_FORMS)
def test_split_ragged_shapes(env, mode):
    shapes = [(1, 1, 1), (2, 3, 5), (33, 17, 9), (130, 70, 65), (127, 63, 129)]
    errs = _grouped(env, mode, shapes, 2)
    assert max(errs) <= SPLIT_TOL, errs


@pytest.mark.parametrize("mode", SPLIT_FORMS)
def test_split_long_k_chunks(env, mode):
    # several 576-k exact-accumulation chunks, drained into double-float
    # (tiled) or 64-bit fixed point (fused); a Gaussian operand
    errs = _grouped(env, mode, [(200, 150, 700), (64, 64, 3000)], 3, dist="normal")
    assert max(errs) <= SPLIT_TOL, errs


def test_split_fused_more_items_than_ctas(env):
    # 16 x 11 + 3 x 2 + 11 = 193 output tiles on at most one CTA per SM: CTAs
    # loop over tiles; K of 200 and 129 walks several 64-k blocks after a
    # scale pass; repeated calls agree bit for bit
    shapes = [(2000, 700, 200), (300, 70, 129), (5, 700, 64)]
    torch, capi, tu = env
    first = _grouped(env, "split_fused", shapes, 6)
    assert max(first) <= SPLIT_TOL, first
    gemms, na, nb, nc = _sectors(shapes)
    rng = np.random.default_rng(7)
    A = torch.from_numpy(rng.uniform(-1, 1, na)).cuda()
    B = torch.from_numpy(rng.uniform(-1, 1, nb)).cuda()
    outs = []
    for _ in range(3):
        Cd = torch.zeros(nc, dtype=torch.float64, device="cuda")
        tu.contract_sectors("split_fused", gemms, A.data_ptr(), B.data_ptr(), Cd.data_ptr())
        tu.sync()
        outs.append(Cd.cpu().numpy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


@pytest.mark.parametrize("mode", SPLIT_FORMS)
def test_split_wide_dynamic_range(env, mode):
    torch, capi, tu = env
    m, n, k = 96, 80, 300
    rng = np.random.default_rng(4)
    a = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-30, 30, (m, 1)))  # rows at very different scales
    b = rng.uniform(-1, 1, (k, n)) * np.exp2(rng.integers(-30, 30, (1, n)))
    A = torch.from_numpy(a.ravel()).cuda()
    B = torch.from_numpy(b.ravel()).cuda()
    Cd = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    tu.contract_sectors(mode, [(m, n, k, 0, 0, 0)], A.data_ptr(), B.data_ptr(), Cd.data_ptr())
    tu.sync()
    c = Cd.cpu().numpy().reshape(m, n)
    want = a @ b
    # per-row/column scaling keeps every entry accurate relative to its row x
    # column scale: each operand carries 49 bits below its row/column maximum,
    # so an entry's error stays under K * 2^-46 of (row max * column max)
    scale = np.abs(a).max(1, keepdims=True) * np.abs(b).max(0, keepdims=True)
    assert np.max(np.abs(c - want) / scale) <= k * 2.0 ** -46
    assert rel(c, want) <= SPLIT_TOL


@pytest.mark.parametrize("mode", ("bf16_tc", "bf16_fused", "bf16_tiled"))
def test_fast_bf16_reports_bf16_level_error(env, mode):
    errs = _grouped(env, mode, [(128, 64, 256), (50, 40, 30)], 5)
    assert max(errs) <= 1e-2, errs


@pytest.mark.parametrize("shapes", [[(128, 64, 256), (50, 40, 30)],
                                    [(1, 1, 1), (33, 17, 9), (130, 70, 65), (127, 63, 129), (300, 200, 600)]])
def test_fast_tf32_reports_tf32_level_error(env, shapes):
    # TF32 keeps 10 mantissa bits (BF16 7): relative error near 2^-11 per
    # operand, accumulated in FP32
    errs = _grouped(env, "tf32_tc", shapes, 6)
    assert max(errs) <= 2e-3, errs
    errs_b = _grouped(env, "bf16_tiled", shapes, 6)
    assert np.mean(errs) < np.mean(errs_b) / 2, (errs, errs_b)


def test_fast_tf32_network(env):
    torch, capi, tu = env
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
        r = net.launch(mode="tf32_tc")
        assert rel(r.get_elem(), G.arr("mera_small", dname)) <= 5e-3, dname


def test_fused_tf32_is_refused(env):
    torch, capi, tu = env
    with pytest.raises(capi.TnError) as e:
        _grouped(env, capi.MODE_FAST_TF32 | capi.MODE_TC_ONLY | capi.MODE_TC_FUSED, [(64, 64, 64)], 1)
    assert e.value.code == 7  # TN_ERR_UNSUPPORTED


def test_split_contract_golden_cases(env):
    torch, capi, tu = env
    for case in [c for c in G.cases().values() if c["kind"] == "contract"]:
        a = tu.UniTensor(G.bonds_of(case["A"]), case["A"]["labels"], G.arr(case["id"], "A"))
        b = tu.UniTensor(G.bonds_of(case["B"]), case["B"]["labels"], G.arr(case["id"], "B"))
        c = tu.contract(a, b, mode="split_tc")
        assert rel(c.get_elem(), G.arr(case["id"], "C")) <= SPLIT_TOL, case["id"]


def test_split_itebd_network(env):
    torch, capi, tu = env
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    net = tu.Network(spec["net"])
    keep = []
    for s in spec["tensors"]:
        t = tu.UniTensor(s.bonds, s.labels, els[s.name])
        keep.append(t)
        net.put_tensor(s.name, t)
    for mode in ("split", "split_tc", "split_fused", "split_tiled"):
        th = net.launch(mode=mode)
        assert rel(th.get_elem(), G.arr("itebd", "TH")) <= SPLIT_TOL, mode


def test_split_mera_and_ipeps_small(env):
    torch, capi, tu = env
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
        r = net.launch(mode="split_tc")
        assert rel(r.get_elem(), G.arr("mera_small", dname)) <= SPLIT_TOL, dname
    c = G.cases()["batched_small"]
    spec = wl.batched(**c["params"])
    for i, (t1, t2) in enumerate(spec["pairs"]):
        a = tu.UniTensor(t1.bonds, t1.labels, G.arr("batched_small", t1.name))
        b = tu.UniTensor(t2.bonds, t2.labels, G.arr("batched_small", t2.name))
        r = tu.contract(a, b, mode="split_tc")
        assert rel(r.get_elem(), G.arr("batched_small", f"C{i}")) <= SPLIT_TOL


def test_network_graph_capture_replay(env):
    """Network::launch recorded as a CUDA graph: replay after new inputs are
    put gives the eager result bit for bit (same kernels, same plans)."""
    torch, capi, tu = env
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    for mode in ("fp64", "split"):
        net = tu.Network(spec["net"])
        ts = {s.name: tu.UniTensor(s.bonds, s.labels, els[s.name]) for s in spec["tensors"]}
        for n, t in ts.items():
            net.put_tensor(n, t)
        net.capture(mode)
        out = net.output()
        eager0 = net.launch(mode).get_elem()
        net.replay()
        assert np.array_equal(out.get_elem(), eager0)
        # new element values in the same tensors: put, replay, compare
        els2 = {n: v * (1.0 + 0.25 * (i + 1)) for i, (n, v) in enumerate(els.items())}
        for n, t in ts.items():
            t.set_elem(els2[n])
            net.put_tensor(n, t)
        net.replay()
        eager = net.launch(mode).get_elem()
        assert np.array_equal(out.get_elem(), eager)
        assert not np.array_equal(eager, eager0)


def test_graph_replay_survives_workspace_growth(env):
    """A captured graph keeps the plans and workspace its kernels read: after
    other work grows the context's workspace (large split-K partials), the
    replay still gives the eager result bit for bit."""
    torch, capi, tu = env
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    net = tu.Network(spec["net"])
    ts = {s.name: tu.UniTensor(s.bonds, s.labels, els[s.name]) for s in spec["tensors"]}
    for n, t in ts.items():
        net.put_tensor(n, t)
    net.capture("fp64")
    out = net.output()
    eager0 = net.launch("fp64").get_elem()
    # the operand slice images of a large split-precision product need far
    # more workspace than the network did
    errs = _grouped(env, "split_tc", [(2048, 2048, 2048)], 9)
    assert max(errs) <= SPLIT_TOL
    net.replay()
    assert np.array_equal(out.get_elem(), eager0)


def test_contract_batch_matches_pairwise(env):
    """One grouped launch for many contractions equals the pairwise contract()
    of each pair: golden fixtures (reference outputs) and 48 random pairs."""
    torch, capi, tu = env
    c = G.cases()["batched_small"]
    spec = wl.batched(**c["params"])
    A = [tu.UniTensor(t1.bonds, t1.labels, G.arr("batched_small", t1.name)) for t1, _ in spec["pairs"]]
    B = [tu.UniTensor(t2.bonds, t2.labels, G.arr("batched_small", t2.name)) for _, t2 in spec["pairs"]]
    for mode, tol in (("fp64", 1e-13), ("split_tc", SPLIT_TOL)):
        outs = tu.contract_batch(A, B, mode)
        for i, o in enumerate(outs):
            assert rel(o.get_elem(), G.arr("batched_small", f"C{i}")) <= tol, (mode, i)
    spec = wl.batched(n=48, lo=16, hi=96, seed=99)
    rng = np.random.default_rng(1)
    A = [tu.UniTensor(t1.bonds, t1.labels, wl.gen_elems(t1, rng)) for t1, _ in spec["pairs"]]
    B = [tu.UniTensor(t2.bonds, t2.labels, wl.gen_elems(t2, rng)) for _, t2 in spec["pairs"]]
    ref = [tu.contract(a, b, mode="fp64").get_elem() for a, b in zip(A, B)]
    for mode, tol in (("fp64", 1e-13), ("split", SPLIT_TOL), ("split_tc", SPLIT_TOL)):
        outs = tu.contract_batch(A, B, mode)
        for o, r in zip(outs, ref):
            assert rel(o.get_elem(), r) <= tol, mode


def test_fused_form_reads_permuted_operands_in_place(env):
    """Where the FP64 kernel reads a permuted operand through views (no permute
    launch), the fused tensor-core form does too; results stay within the
    split tolerance of the reference's outputs, and a contraction whose
    operands need no permute gives the same numbers through either path."""
    torch, capi, tu = env
    seen_views = 0
    for case in [c for c in G.cases().values() if c["kind"] == "contract"]:
        a = tu.UniTensor(G.bonds_of(case["A"]), case["A"]["labels"], G.arr(case["id"], "A"))
        b = tu.UniTensor(G.bonds_of(case["B"]), case["B"]["labels"], G.arr(case["id"], "B"))
        counts = {}
        for mode in ("fp64", "split_fused"):
            tu.prof_enable(True)
            c = tu.contract(a, b, mode=mode)
            prof = tu.prof_read()
            tu.prof_enable(False)
            counts[mode] = prof.get("permute", {}).get("launches", 0)
            tol = 1e-13 if mode == "fp64" else SPLIT_TOL
            assert rel(c.get_elem(), G.arr(case["id"], "C")) <= tol, (case["id"], mode)
        assert counts["split_fused"] <= counts["fp64"], (case["id"], counts)
        seen_views += counts["fp64"] == 0
    assert seen_views > 0


def test_graph_host_io_odd_counts_and_8_byte_offsets(env):
    """Host-bound graph I/O where the one-launch copy list takes its 8-byte
    path (a host buffer 8 bytes past a 16-byte boundary) and its odd-count
    tail (15, 35 and 21 elements): the replayed result is the product of the
    current host inputs, bit-identical to an eager launch."""
    torch, capi, tu = env
    net = tu.Network("X: 1; 2\nY: 2; 3\nTOUT: 1; 3\n")
    dims = {"X": (3, 5), "Y": (5, 7)}
    bond = lambda t, d: wl.u1_bond(t, (0,), (d,))
    rng = np.random.default_rng(7)
    els = {n: rng.uniform(-1, 1, m * k) for n, (m, k) in dims.items()}
    ts = {"X": tu.UniTensor([bond(wl.IN, 3), bond(wl.OUT, 5)], [1, 2], els["X"]),
          "Y": tu.UniTensor([bond(wl.IN, 5), bond(wl.OUT, 7)], [2, 3], els["Y"])}
    for n, t in ts.items():
        net.put_tensor(n, t)
    eager = net.launch("fp64").get_elem()
    want = els["X"].reshape(3, 5) @ els["Y"].reshape(5, 7)
    assert np.abs(eager - want.ravel()).max() <= 1e-13 * np.abs(want).max()
    # X one element into its pinned buffer (8-byte aligned only), Y at the start
    xbuf = torch.zeros(16 + 1, dtype=torch.float64).pin_memory()
    xbuf[1:16].copy_(torch.from_numpy(els["X"]))
    ybuf = torch.from_numpy(els["Y"].copy()).pin_memory()
    obuf = torch.full((22,), np.nan, dtype=torch.float64).pin_memory()
    net.bind_host_input("X", xbuf.data_ptr() + 8, 15)
    net.bind_host_input("Y", ybuf.data_ptr(), 35)
    net.bind_host_output(obuf.data_ptr() + 8, 21)
    net.capture("fp64")
    net.replay()
    tu.sync()
    assert np.array_equal(obuf[1:].numpy(), eager)
    assert np.isnan(obuf[0].item())  # nothing written before the bound output
    xbuf[1:16].mul_(-2.0)
    ybuf.add_(0.5)
    net.replay()
    tu.sync()
    ts["X"].set_elem(xbuf[1:16].numpy().copy())
    ts["Y"].set_elem(ybuf.numpy().copy())
    for n, t in ts.items():
        net.put_tensor(n, t)
    assert np.array_equal(obuf[1:].numpy(), net.launch("fp64").get_elem())


def test_graph_with_host_bound_inputs_and_output(env):
    """Network capture with pinned host buffers bound: every replay copies the
    current host inputs in and theta out; bit-identical to eager launches on
    the same values, and it follows new host contents."""
    torch, capi, tu = env
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    net = tu.Network(spec["net"])
    ts = {s.name: tu.UniTensor(s.bonds, s.labels, els[s.name]) for s in spec["tensors"]}
    for n, t in ts.items():
        net.put_tensor(n, t)
    for mode in ("fp64", "split"):
        eager = net.launch(mode).get_elem()
        pinned = {n: torch.from_numpy(v.copy()).pin_memory() for n, v in els.items()}
        out = torch.full((eager.size,), np.nan, dtype=torch.float64).pin_memory()
        for n in ts:
            net.bind_host_input(n, pinned[n].data_ptr(), els[n].size)
        net.bind_host_output(out.data_ptr(), eager.size)
        net.capture(mode)
        net.replay()
        tu.sync()
        assert np.array_equal(out.numpy(), eager), mode
        for i, n in enumerate(ts):
            pinned[n].mul_(1.0 + 0.25 * (i + 1))
        net.replay()
        tu.sync()
        for n, t in ts.items():
            t.set_elem(pinned[n].numpy())
            net.put_tensor(n, t)
        eager2 = net.launch(mode).get_elem()
        assert np.array_equal(out.numpy(), eager2), mode
        assert not np.array_equal(eager2, eager)
        for n, t in ts.items():  # back to the original values for the next mode
            t.set_elem(els[n])
            net.put_tensor(n, t)
