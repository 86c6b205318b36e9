"""Seeded synthetic inputs for the five block-tensor workloads.

A bond is ``(btype, [(u1, prt, prtf, deg), ...])`` with ``btype`` +1 (IN) or
-1 (OUT) -- the run-length form of a uni10 Bond.  A tensor spec is
``TensorSpec(name, bonds, labels)``; its elements are drawn in elem order
(blocks in Qnum order, each row-major), which is what ``setElem`` takes, so the
same array feeds the GPU path and the CPU checker.

Workloads (every input synthetic; no dataset is involved):
  1. ``u1_rank4``   -- rank-4 U(1) A[a,p,q,b] and B[b,q,r,c], chi=64, charges -3..3
  2. ``itebd``      -- one iTEBD step, spin-1/2 Heisenberg with U(1) Sz, chi=512
  3. ``ipeps_ctm``  -- Z2 iPEPS double-layer CTM quadrant, chi=128, D=8
  4. ``batched``    -- 1024 uneven U(1) rank-3 x rank-3 contractions
  5. ``mera``       -- dense ternary MERA ascending superoperator, chi=24
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

IN, OUT = 1, -1
EVEN, ODD = 0, 1


@dataclass
class TensorSpec:
    name: str
    bonds: list
    labels: list
    kind: str = "uniform"  # uniform | normal | diag | given
    extra: dict = field(default_factory=dict)


def u1_bond(btype, charges, degs):
    return (btype, [(int(q), 0, 0, int(d)) for q, d in zip(charges, degs) if d > 0])


def z2_bond(btype, n_even, n_odd):
    runs = []
    if n_even:
        runs.append((0, EVEN, 0, n_even))
    if n_odd:
        runs.append((0, ODD, 0, n_odd))
    return (btype, runs)


def dense_bond(btype, dim):
    return (btype, [(0, 0, 0, dim)])


def _qkey(q):
    return q[0] * 4 + q[1] * 2 + q[2]


def _fuse(a, b):
    return (a[0] + b[0], a[1] ^ b[1], a[2] ^ b[2])


def _neg(q):
    return (-q[0], q[1], q[2])


def change(bond, btype):
    """Bond::change: flip direction and negate charges."""
    t, runs = bond
    if t == btype:
        return bond
    return (btype, [(-u, p, f, d) for (u, p, f, d) in runs])


def combine2(b1, b2):
    """Bond::combine (b1 keeps its type; b2 is changed to it first)."""
    t = b1[0]
    b2 = change(b2, t)
    runs = []
    for (u, p, f, d) in b1[1]:
        for _ in range(d):
            for (u2, p2, f2, d2) in b2[1]:
                q = _fuse((u, p, f), (u2, p2, f2))
                if runs and runs[-1][:3] == q:
                    runs[-1] = (*q, runs[-1][3] + d2)
                else:
                    runs.append((*q, d2))
    return (t, runs)


def combine(btype, bonds):
    """combine(bondType, vector<Bond>): right-to-left fold."""
    if len(bonds) == 1:
        return change(bonds[0], btype)
    out = change(bonds[-2], btype)
    out = combine2(out, bonds[-1])
    for b in range(len(bonds) - 3, -1, -1):
        out = combine2(change(bonds[b], btype), out)
    return out


def _hist(bonds):
    h = {(0, 0, 0): 1}
    for (_, runs) in bonds:
        nh = {}
        for q, n in h.items():
            for (u, p, f, d) in runs:
                k = _fuse(q, (u, p, f))
                nh[k] = nh.get(k, 0) + n * d
        h = nh
    return h


def elem_count(bonds) -> int:
    """Number of stored elements: sum over charges present on both sides of
    rows(q) * cols(q), rows from the IN bonds, cols from the OUT bonds."""
    rows = [b for b in bonds if b[0] == IN]
    cols = [b for b in bonds if b[0] == OUT]
    r = _hist(rows)
    c = _hist(cols)
    return int(sum(r[q] * c[q] for q in r if q in c))


def block_shapes(bonds):
    """[(qnum, rows, cols)] in block (Qnum) order."""
    rows = [b for b in bonds if b[0] == IN]
    cols = [b for b in bonds if b[0] == OUT]
    r, c = _hist(rows), _hist(cols)
    return [(q, r[q], c[q]) for q in sorted((q for q in r if q in c), key=_qkey)]


def diag_blocks(bonds, elems):
    """[(qnum, rows, cols, diagonal)] of a tensor whose blocks are diagonal,
    read from its elements in block order (what putBlock with diagonal
    matrices rebuilds)."""
    out, off = [], 0
    for q, r, c in block_shapes(bonds):
        blk = np.asarray(elems[off : off + r * c]).reshape(r, c)
        out.append((q, r, c, np.diagonal(blk).copy()))
        off += r * c
    return out


def gen_elems(spec: TensorSpec, rng: np.random.Generator) -> np.ndarray:
    n = elem_count(spec.bonds)
    if spec.kind == "uniform":
        return rng.uniform(-1.0, 1.0, n)
    if spec.kind == "normal":
        return rng.standard_normal(n)
    if spec.kind == "diag":  # block-diagonal positive, sorted descending per block
        out = np.zeros(n)
        off = 0
        for q, r, c in block_shapes(spec.bonds):
            v = np.sort(rng.uniform(0.1, 1.0, r))[::-1]
            blk = np.zeros((r, c))
            blk[np.arange(r), np.arange(r)] = v
            out[off : off + r * c] = blk.ravel()
            off += r * c
        return out
    if spec.kind == "given":
        return np.asarray(spec.extra["elems"], dtype=np.float64)
    raise ValueError(spec.kind)


# ------------------------------------------------------------------ workload 1
CHI64_DEGS = (2, 6, 12, 24, 12, 6, 2)


def u1_rank4():
    """A[a,p,q,b] (a,p,q IN; b OUT), B[b,q,r,c] (b,q IN; r,c OUT); a,b,c dim 64
    over U(1) charges -3..3, p,q,r charges (+1,-1).  Permute A to (a,p,b,q)
    with 2 in-bonds, then contract over b,q."""
    v = lambda t: u1_bond(t, range(-3, 4), CHI64_DEGS)
    s = lambda t: u1_bond(t, (1, -1), (1, 1))
    a = TensorSpec("A", [v(IN), s(IN), s(IN), v(OUT)], [0, 1, 2, 3])
    b = TensorSpec("B", [v(IN), s(IN), s(OUT), v(OUT)], [3, 2, 4, 5])
    return {"tensors": [a, b], "seed": 1001, "permute": ("A", [0, 1, 3, 2], 2)}


# ------------------------------------------------------------------ workload 2
ITEBD_DEGS = (2, 5, 9, 17, 28, 41, 55, 65, 68, 65, 55, 41, 28, 17, 9, 5, 2)
ITEBD_NET = """La: -1; 10
A: 10 1; 11
Lb: 11; 12
B: 12 2; 13
Lc: 13; -3
U: -2 -4; 1 2
TOUT: -1 -2; -4 -3
ORDER: (((((La A) Lb) B) Lc) U)
"""


def heisenberg_gate_blocks(tau: float = 0.01):
    """exp(-tau H) for H = S1.S2 (spin-1/2) in U(1) blocks of total 2*Sz:
    +2 and -2 are 1x1, 0 is 2x2 over (up,down), (down,up)."""
    h0 = np.array([[-0.25, 0.5], [0.5, -0.25]])
    w, v = np.linalg.eigh(h0)
    g0 = (v * np.exp(-tau * w)) @ v.T
    gp = np.array([[np.exp(-tau * 0.25)]])
    return {-2: gp, 0: g0, 2: gp}


def itebd(chi_degs=ITEBD_DEGS, tau: float = 0.01):
    """One iTEBD step: La-A-Lb-B-Lc-U contracted to theta[a,s1'|s2',c]."""
    ch = range(-(len(chi_degs) // 2), len(chi_degs) // 2 + 1)
    v = lambda t: u1_bond(t, ch, chi_degs)
    s = lambda t: u1_bond(t, (1, -1), (1, 1))
    La = TensorSpec("La", [v(IN), v(OUT)], [-1, 10], kind="diag")
    A = TensorSpec("A", [v(IN), s(IN), v(OUT)], [10, 1, 11])
    Lb = TensorSpec("Lb", [v(IN), v(OUT)], [11, 12], kind="diag")
    B = TensorSpec("B", [v(IN), s(IN), v(OUT)], [12, 2, 13])
    Lc = TensorSpec("Lc", [v(IN), v(OUT)], [13, -3], kind="diag")
    ubonds = [s(IN), s(IN), s(OUT), s(OUT)]
    g = heisenberg_gate_blocks(tau)
    # gate elements in block order: charges -2, 0, +2 (row-major blocks)
    gel = np.concatenate([g[q].ravel() for q in (-2, 0, 2)])
    U = TensorSpec("U", ubonds, [-2, -4, 1, 2], kind="given", extra={"elems": gel})
    return {"tensors": [La, A, Lb, B, Lc, U], "seed": 2002, "net": ITEBD_NET, "chi": int(sum(chi_degs))}


# ------------------------------------------------------------------ workload 3
IPEPS_NET = """C: 1; 2
T1: 2 10; 3
T2: 4 20; 1
A2: 10 20; 30 40
TOUT: 3 4; 30 40
ORDER: (((C T1) T2) A2)
"""


def ipeps_ctm(chi: int = 128, D: int = 8, d: int = 2):
    """Z2 iPEPS CTM quadrant.  Site a[p|u,l,d,r] (d=2: 1 even + 1 odd; D=8:
    4 even + 4 odd), entries N(0,1).  The double-layer A2 = a.a* over p with
    the (x, x') pairs combined (D^2=64 per leg) is built on the device from a.
    C[chi|chi], T1[chi,D^2|chi], T2[chi,D^2|chi], chi = chi/2 even + chi/2 odd."""
    p = z2_bond(IN, d // 2, d - d // 2)
    vD = lambda t: z2_bond(t, D // 2, D - D // 2)
    site = TensorSpec("a", [p, vD(OUT), vD(OUT), vD(OUT), vD(OUT)], [0, 1, 2, 3, 4], kind="normal")
    dd = combine(IN, [vD(IN), vD(OUT)])  # the combined double-layer leg
    c = lambda t: z2_bond(t, chi // 2, chi - chi // 2)
    C = TensorSpec("C", [c(IN), c(OUT)], [1, 2], kind="normal")
    T1 = TensorSpec("T1", [c(IN), dd, c(OUT)], [2, 10, 3], kind="normal")
    T2 = TensorSpec("T2", [c(IN), dd, c(OUT)], [4, 20, 1], kind="normal")
    return {"tensors": [site, C, T1, T2], "seed": 3003, "net": IPEPS_NET}


# ------------------------------------------------------------------ workload 4
def _dirichlet_degs(rng, dim, ncharge):
    w = rng.dirichlet(np.ones(ncharge)) * dim
    base = np.floor(w).astype(int)
    rem = dim - base.sum()
    order = np.argsort(-(w - base), kind="stable")
    base[order[:rem]] += 1
    return base


def batched(n: int = 1024, lo: int = 16, hi: int = 256, seed: int = 4004):
    """n independent U(1) contractions T1[x|y,z] . T2[y,z|w] over (y,z).
    Every bond dim ~ U{lo..hi}; charges -4..4 with Dirichlet(1) degeneracies
    rounded to integers summing to the dim (zero-degeneracy charges dropped)."""
    rng = np.random.default_rng(seed)
    charges = np.arange(-4, 5)
    pairs = []
    for i in range(n):
        dims = rng.integers(lo, hi + 1, size=4)
        degs = [_dirichlet_degs(rng, int(dm), len(charges)) for dm in dims]
        x, y, z, w = (lambda t, dg=dg: u1_bond(t, charges, dg) for dg in degs)
        t1 = TensorSpec(f"T1_{i}", [x(IN), y(OUT), z(OUT)], [0, 1, 2])
        t2 = TensorSpec(f"T2_{i}", [y(IN), z(IN), w(OUT)], [1, 2, 3])
        pairs.append((t1, t2))
    return {"pairs": pairs, "seed": seed + 1}


# ------------------------------------------------------------------ workload 5
def qr_isometry(rng, rows, cols):
    g = rng.standard_normal((rows, cols))
    q, r = np.linalg.qr(g)
    return q * np.sign(np.diag(r))


# Ternary MERA, 3-site operators: isometry w[i1,i2,i3 | o] (three lower legs
# in, one upper leg out), disentangler u[i1,i2 | o1,o2] (lower legs in).  The
# operator O[s1,s2,s3 | t1,t2,t3] lives on three consecutive lower sites.  In
# each diagram two isometries (W1 over lower sites 0..2, W2 over 3..5) and one
# disentangler U on sites (2,3) form the ket layer above O; the same tensors,
# mirrored (Ud, W1d, W2d), form the bra layer below.  Lower sites that O does
# not touch are traced straight through.
#   left   diagram: O on sites (1,2,3)
#   center diagram: O on sites (2,3,4)
#   right  diagram: O on sites (3,4,5)
# Each maps O to a 2-site operator on the isometries' upper legs; the ORDER
# lines keep every pairwise step at chi^8 multiply-adds or fewer (3-4 such
# steps per diagram, chi^6 intermediates).
MERA_NETS = {
    "left": """W1: 1 2 3; 100
W2: 4 5 6; 200
U: 13 14; 3 4
O: 22 23 24; 2 13 14
Ud: 23 24; 33 34
W1d: 1 22 33; 101
W2d: 34 5 6; 201
TOUT: 101 201; 100 200
ORDER: (((((U O) Ud) W1) W1d) (W2 W2d))
""",
    "center": """W1: 1 2 3; 100
W2: 4 5 6; 200
U: 13 14; 3 4
O: 23 24 25; 13 14 5
Ud: 23 24; 33 34
W1d: 1 2 33; 101
W2d: 34 25 6; 201
TOUT: 101 201; 100 200
ORDER: (((((U O) Ud) (W1 W1d)) W2) W2d)
""",
    "right": """W1: 1 2 3; 100
W2: 4 5 6; 200
U: 13 14; 3 4
O: 24 25 26; 14 5 6
Ud: 13 24; 33 34
W1d: 1 2 33; 101
W2d: 34 25 26; 201
TOUT: 101 201; 100 200
ORDER: (((O W2) W2d) ((U Ud) (W1 W1d)))
""",
}


def mera(chi: int = 24, seed: int = 5005):
    """Dense ternary MERA ascending superoperator, no symmetry (one sector).
    w, u from QR of seeded N(0,1) matrices (isometric); O = (G+G^T)/2 with G
    iid N(0,1), a chi^3 x chi^3 Hermitian (real symmetric) operator."""
    rng = np.random.default_rng(seed)
    b = lambda t: dense_bond(t, chi)
    w = qr_isometry(rng, chi ** 3, chi)  # columns orthonormal: w^T w = 1
    u = qr_isometry(rng, chi ** 2, chi ** 2)
    g = rng.standard_normal((chi ** 3, chi ** 3))
    o = 0.5 * (g + g.T)
    del g
    W = lambda n: TensorSpec(n, [b(IN), b(IN), b(IN), b(OUT)], [0, 1, 2, 3], kind="given", extra={"elems": w.ravel()})
    # u[i1,i2|o1,o2]: rows are lower legs; an orthogonal chi^2 x chi^2 matrix
    U = lambda n: TensorSpec(n, [b(IN), b(IN), b(OUT), b(OUT)], [0, 1, 2, 3], kind="given", extra={"elems": u.ravel()})
    O = TensorSpec("O", [b(IN)] * 3 + [b(OUT)] * 3, list(range(6)), kind="given", extra={"elems": o.ravel()})
    return {"tensors": [W("W1"), W("W2"), U("U"), O, U("Ud"), W("W1d"), W("W2d")], "nets": MERA_NETS, "seed": seed}


def bond_dims(bond) -> int:
    return int(sum(r[3] for r in bond[1]))
