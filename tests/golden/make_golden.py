"""Generate the golden fixtures in this directory from the compiled reference.

Run here (where the reference sources exist and oracle/_ref is built):

    make -C oracle/refbuild REFSRC=<reference project root>/uni10/src
    python tests/golden/make_golden.py --refroot <reference project root>/uni10

It writes:
  cases.json / arrays.npz  reference outputs (UniTensor::permute, transpose,
                           contract, combineBond, Network::launch, Block::svd,
                           Block::eigh, UniTensor::addGate, fermionic
                           Network::launch with swap gates)
                           for seeded inputs: workload 1 at full size, the
                           iTEBD network at full size (chi=512), reduced-size
                           versions of workloads 3-5, and randomized
                           signatures.  Inputs are stored for the small cases;
                           the large ones store the SHA-256 of their seeded
                           inputs so a test can tell an RNG drift from a bug.
  legacy.npz               the reference's own fixtures Swig/examples/egU3_W,
                           egU3_WT, egU1_H_U1 and mat_U/mat_Sigma/mat_VT,
                           decoded from their legacy binary layout (with the
                           SHA-256 of each file's bytes, which pins the
                           legacy writer of oracle/uni10_io.py).
  saved/*.uni10, saved.json  tensors written by the reference's
                           UniTensor::save (current layout) from seeded
                           inputs, for the product's file reader.

    python tests/golden/make_golden.py --refroot ... --only saved,legacy
regenerates only the last two.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refrun, uni10_io  # noqa: E402
from trim_gb300 import workloads as wl  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


class Writer:
    def __init__(self):
        self.cases = []
        self.arrays = {}

    def add(self, case: dict, arrays: dict):
        for k, v in arrays.items():
            self.arrays[f"{case['id']}/{k}"] = v
        self.cases.append(case)


def tensor_meta(bonds, labels):
    return {"bonds": [[t, [list(r) for r in runs]] for t, runs in bonds], "labels": list(labels)}


def out_meta(d):
    return {"bonds": [[t, [list(r) for r in runs]] for t, runs in d["bonds"]], "labels": d["labels"], "sha256": sha(d["elem"]), "n": int(d["elem"].size)}


# ---------------------------------------------------------------- random signatures
def rand_bond(rng, btype, sym):
    if sym == "u1":
        nq = int(rng.integers(1, 4))
        qs = rng.choice(np.arange(-2, 3), size=nq, replace=False)
        return (btype, [(int(q), 0, 0, int(rng.integers(1, 4))) for q in qs])
    if sym == "z2":
        runs = []
        for p in rng.permutation(2)[: int(rng.integers(1, 3))]:
            runs.append((0, int(p), 0, int(rng.integers(1, 4))))
        return (btype, runs)
    if sym == "fermion":  # U(1) charges with fermionic parity (PRTF_ODD sets the reference's Fermionic flag)
        pool = [(-1, 0), (-1, 1), (0, 0), (0, 1), (1, 0), (1, 1)]
        nq = int(rng.integers(1, 4))
        pick = sorted(rng.choice(len(pool), size=nq, replace=False))
        return (btype, [(pool[k][0], 0, pool[k][1], int(rng.integers(1, 4))) for k in pick])
    if sym == "fermion_rich":  # 2-4 charges, at least one of odd fermionic parity
        pool = [(-1, 0), (-1, 1), (0, 0), (0, 1), (1, 0), (1, 1)]
        while True:
            pick = sorted(rng.choice(len(pool), size=int(rng.integers(2, 5)), replace=False))
            if any(pool[k][1] for k in pick):
                return (btype, [(pool[k][0], 0, pool[k][1], int(rng.integers(1, 4))) for k in pick])
    return (btype, [(0, 0, 0, int(rng.integers(1, 5)))])


def rand_tensor(rng, rank, sym):
    nin = int(rng.integers(0, rank + 1))
    while True:
        bonds = [rand_bond(rng, 1 if i < nin else -1, sym) for i in range(rank)]
        if wl.elem_count(bonds) > 0:
            return bonds


def permute_cases(w: Writer, rng, n: int):
    for i in range(n):
        sym = ["u1", "z2", "dense", "u1", "u1"][i % 5]
        rank = int(rng.integers(2, 7))
        bonds = rand_tensor(rng, rank, sym)
        labels = list(rng.permutation(np.arange(10, 10 + rank)))
        labels = [int(x) for x in labels]
        perm = [labels[j] for j in rng.permutation(rank)]
        rn = int(rng.integers(0, rank + 1))
        el = rng.uniform(-1, 1, wl.elem_count(bonds))
        S = refrun.RefSession()
        S.tensor("T", bonds, labels, el)
        S.cmd(f"permute T {rn} " + " ".join(map(str, perm)))
        S.save("T", "P")
        S.cmd("transpose T")
        S.save("T", "PT")
        o = S.run()
        case = {"id": f"perm{i}", "kind": "permute", "T": tensor_meta(bonds, labels), "new_labels": perm, "rownum": rn,
                "out": out_meta(o["P"]), "out_transpose": out_meta(o["PT"])}
        w.add(case, {"T": el, "P": o["P"]["elem"], "PT": o["PT"]["elem"]})


def contract_cases(w: Writer, rng, n: int):
    """Random pairs sharing 1..3 bonds (opposite directions), random label order."""
    made = 0
    while made < n:
        sym = ["u1", "z2", "dense"][made % 3]
        nfa, nfb, nsh = int(rng.integers(0, 3)), int(rng.integers(0, 3)), int(rng.integers(1, 4))
        shared = [rand_bond(rng, -1, sym) for _ in range(nsh)]
        fa = [rand_bond(rng, 1, sym) for _ in range(nfa)]
        fb = [rand_bond(rng, -1, sym) for _ in range(nfb)]
        a_bonds = fa + shared
        b_bonds = [wl.change(s, 1) for s in shared] + fb
        if wl.elem_count(a_bonds) == 0 or wl.elem_count(b_bonds) == 0:
            continue
        la = list(range(100, 100 + nfa)) + list(range(200, 200 + nsh))
        lb = list(range(200, 200 + nsh)) + list(range(300, 300 + nfb))
        ea = rng.uniform(-1, 1, wl.elem_count(a_bonds))
        eb = rng.uniform(-1, 1, wl.elem_count(b_bonds))
        # scramble the operands' bond order (as a user tensor would come)
        pa = [la[j] for j in rng.permutation(len(la))]
        pb = [lb[j] for j in rng.permutation(len(lb))]
        ra, rb = int(rng.integers(0, len(la) + 1)), int(rng.integers(0, len(lb) + 1))
        S = refrun.RefSession()
        S.tensor("A", a_bonds, la, ea)
        S.tensor("B", b_bonds, lb, eb)
        S.cmd(f"permute A {ra} " + " ".join(map(str, pa)))
        S.cmd(f"permute B {rb} " + " ".join(map(str, pb)))
        S.save("A", "A1")
        S.save("B", "B1")
        S.cmd("contract C A B 0")
        S.save("C")
        try:
            o = S.run()
        except RuntimeError:
            continue
        if "C" not in o:
            continue
        case = {"id": f"con{made}", "kind": "contract", "A": tensor_meta(o["A1"]["bonds"], o["A1"]["labels"]),
                "B": tensor_meta(o["B1"]["bonds"], o["B1"]["labels"]), "out": out_meta(o["C"])}
        w.add(case, {"A": o["A1"]["elem"], "B": o["B1"]["elem"], "C": o["C"]["elem"]})
        made += 1


def fermion_cases(w: Writer, rng, nperm: int, ncon: int):
    """Permutes and contractions of tensors with fermionic charges: the
    reference multiplies each moved sub-block by its swap sign."""
    made = 0
    while made < nperm:
        rank = int(rng.integers(2, 7))
        bonds = rand_tensor(rng, rank, "fermion")
        if all(len(runs) == 1 for _, runs in bonds):
            continue  # a single charge per bond takes the reference's dense path
        labels = [int(x) for x in rng.permutation(np.arange(10, 10 + rank))]
        perm = [labels[j] for j in rng.permutation(rank)]
        rn = int(rng.integers(0, rank + 1))
        el = rng.uniform(-1, 1, wl.elem_count(bonds))
        S = refrun.RefSession()
        S.tensor("T", bonds, labels, el)
        S.cmd(f"permute T {rn} " + " ".join(map(str, perm)))
        S.save("T", "P")
        S.cmd("transpose T")
        S.save("T", "PT")
        o = S.run()
        case = {"id": f"fperm{made}", "kind": "permute", "T": tensor_meta(bonds, labels), "new_labels": perm,
                "rownum": rn, "out": out_meta(o["P"]), "out_transpose": out_meta(o["PT"])}
        w.add(case, {"T": el, "P": o["P"]["elem"], "PT": o["PT"]["elem"]})
        made += 1
    made = 0
    while made < ncon:
        nfa, nfb, nsh = int(rng.integers(1, 3)), int(rng.integers(1, 3)), int(rng.integers(1, 3))
        shared = [rand_bond(rng, -1, "fermion") for _ in range(nsh)]
        fa = [rand_bond(rng, 1, "fermion") for _ in range(nfa)]
        fb = [rand_bond(rng, -1, "fermion") for _ in range(nfb)]
        a_bonds = fa + shared
        b_bonds = [wl.change(x, 1) for x in shared] + fb
        if wl.elem_count(a_bonds) == 0 or wl.elem_count(b_bonds) == 0:
            continue
        la = list(range(100, 100 + nfa)) + list(range(200, 200 + nsh))
        lb = list(range(200, 200 + nsh)) + list(range(300, 300 + nfb))
        ea = rng.uniform(-1, 1, wl.elem_count(a_bonds))
        eb = rng.uniform(-1, 1, wl.elem_count(b_bonds))
        pa = [la[j] for j in rng.permutation(len(la))]
        pb = [lb[j] for j in rng.permutation(len(lb))]
        ra, rb = int(rng.integers(0, len(la) + 1)), int(rng.integers(0, len(lb) + 1))
        S = refrun.RefSession()
        S.tensor("A", a_bonds, la, ea)
        S.tensor("B", b_bonds, lb, eb)
        S.cmd(f"permute A {ra} " + " ".join(map(str, pa)))
        S.cmd(f"permute B {rb} " + " ".join(map(str, pb)))
        S.save("A", "A1")
        S.save("B", "B1")
        S.cmd("contract C A B 0")
        S.save("C")
        try:
            o = S.run()
        except RuntimeError:
            continue
        if "C" not in o:
            continue
        case = {"id": f"fcon{made}", "kind": "contract", "A": tensor_meta(o["A1"]["bonds"], o["A1"]["labels"]),
                "B": tensor_meta(o["B1"]["bonds"], o["B1"]["labels"]), "out": out_meta(o["C"])}
        w.add(case, {"A": o["A1"]["elem"], "B": o["B1"]["elem"], "C": o["C"]["elem"]})
        made += 1


# ---------------------------------------------------------------- workloads
def run_tensors(S, specs, rng):
    els = {}
    for s in specs:
        els[s.name] = wl.gen_elems(s, rng)
        S.tensor(s.name, s.bonds, s.labels, els[s.name])
    return els


def workload1(w: Writer):
    spec = wl.u1_rank4()
    rng = np.random.default_rng(spec["seed"])
    S = refrun.RefSession()
    els = run_tensors(S, spec["tensors"], rng)
    name, labs, rn = spec["permute"]
    S.cmd(f"permute {name} {rn} " + " ".join(map(str, labs)))
    S.save("A", "PA")
    S.cmd("contract C A B 0")
    S.save("C")
    o = S.run()
    case = {"id": "u1_rank4", "kind": "workload", "inputs_sha": {k: sha(v) for k, v in els.items()},
            "PA": out_meta(o["PA"]), "C": out_meta(o["C"])}
    w.add(case, {"A": els["A"], "B": els["B"], "PA": o["PA"]["elem"], "C": o["C"]["elem"]})


def workload2(w: Writer):
    spec = wl.itebd()
    rng = np.random.default_rng(spec["seed"])
    S = refrun.RefSession()
    els = run_tensors(S, spec["tensors"], rng)
    S.network("TH", spec["net"], {s.name: s.name for s in spec["tensors"]})
    S.save("TH")
    o = S.run()
    th = o["TH"]
    # per-sector singular values of theta (Block::svd -> dgesvd)
    blocks = wl.block_shapes(th["bonds"])
    S2 = refrun.RefSession()
    S2.tensor("TH", th["bonds"], th["labels"], th["elem"])
    for i, (q, r, c) in enumerate(blocks):
        S2.svd("TH", q, f"s{i}")
    o2 = S2.run()
    svals = np.concatenate([np.atleast_1d(o2[f"s{i}"][1]).ravel() for i in range(len(blocks))])
    case = {"id": "itebd", "kind": "workload", "inputs_sha": {k: sha(v) for k, v in els.items()},
            "TH": out_meta(th), "svd_blocks": [[list(q), r, c] for q, r, c in blocks]}
    w.add(case, {"TH": th["elem"], "S": svals})


def workload3_small(w: Writer):
    spec = wl.ipeps_ctm(chi=16, D=4)
    rng = np.random.default_rng(spec["seed"])
    site, C, T1, T2 = spec["tensors"]
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    S = refrun.RefSession()
    for s in spec["tensors"]:
        S.tensor(s.name, s.bonds, s.labels, els[s.name])
    # double layer: a (p,u,l,d,r) . a* (p,u',l',d',r') over p, then combine (x,x')
    S.cmd("copy ac a")
    S.cmd("labels ac 0 11 12 13 14")
    S.cmd("contract aa a ac 0")
    for x in (1, 2, 3, 4):
        S.cmd(f"combine aa {x} {x + 10}")
    S.cmd("permute_rows aa 2")
    S.save("aa", "AA")
    o = S.run()
    aa = o["AA"]
    S2 = refrun.RefSession()
    for s in (C, T1, T2):
        S2.tensor(s.name, s.bonds, s.labels, els[s.name])
    S2.tensor("A2", aa["bonds"], [10, 20, 30, 40], aa["elem"])
    S2.network("Q", spec["net"], {"C": "C", "T1": "T1", "T2": "T2", "A2": "A2"})
    S2.save("Q")
    o2 = S2.run()
    case = {"id": "ipeps_small", "kind": "workload", "params": {"chi": 16, "D": 4}, "AA": out_meta(aa), "Q": out_meta(o2["Q"])}
    w.add(case, {**{k: v for k, v in els.items()}, "AA": aa["elem"], "Q": o2["Q"]["elem"]})


def workload4_small(w: Writer):
    spec = wl.batched(n=6, lo=4, hi=24, seed=77)
    rng = np.random.default_rng(spec["seed"])
    S = refrun.RefSession()
    arrays = {}
    for i, (t1, t2) in enumerate(spec["pairs"]):
        e1, e2 = wl.gen_elems(t1, rng), wl.gen_elems(t2, rng)
        S.tensor(t1.name, t1.bonds, t1.labels, e1)
        S.tensor(t2.name, t2.bonds, t2.labels, e2)
        S.cmd(f"contract C{i} {t1.name} {t2.name} 0")
        S.save(f"C{i}")
        arrays[t1.name], arrays[t2.name] = e1, e2
    o = S.run()
    outs = {}
    for i in range(len(spec["pairs"])):
        arrays[f"C{i}"] = o[f"C{i}"]["elem"]
        outs[f"C{i}"] = out_meta(o[f"C{i}"])
    w.add({"id": "batched_small", "kind": "workload", "params": {"n": 6, "lo": 4, "hi": 24, "seed": 77}, "outs": outs}, arrays)


def workload5_small(w: Writer):
    spec = wl.mera(chi=4, seed=505)
    rng = np.random.default_rng(0)
    els = {s.name: wl.gen_elems(s, rng) for s in spec["tensors"]}
    arrays = {}
    outs = {}
    for dname, net in spec["nets"].items():
        S = refrun.RefSession()
        for s in spec["tensors"]:
            S.tensor(s.name, s.bonds, s.labels, els[s.name])
        S.network("R", net, {s.name: s.name for s in spec["tensors"]})
        S.save("R")
        o = S.run()
        arrays[dname] = o["R"]["elem"]
        outs[dname] = out_meta(o["R"])
    w.add({"id": "mera_small", "kind": "workload", "params": {"chi": 4, "seed": 505}, "outs": outs}, arrays)


GREEDY_NET = """A: 1 2; 3
B: 3 4; 5
C: 5; 6 7
D: 2 7; 8
TOUT: 1 4; 6 8
"""


def greedy_network(w: Writer, rng):
    """No ORDER line: the tree comes from the reference's greedy planner."""
    d = lambda t: (t, [(0, 0, 0, int(rng.integers(2, 6)))])
    b1, b2, b3, b4, b5, b6, b7, b8 = (int(rng.integers(2, 6)) for _ in range(8))
    mk = lambda t, n: (t, [(0, 0, 0, n)])
    specs = {
        "A": [mk(1, b1), mk(1, b2), mk(-1, b3)],
        "B": [mk(1, b3), mk(1, b4), mk(-1, b5)],
        "C": [mk(1, b5), mk(-1, b6), mk(-1, b7)],
        "D": [mk(1, b2), mk(1, b7), mk(-1, b8)],
    }
    labels = {"A": [1, 2, 3], "B": [3, 4, 5], "C": [5, 6, 7], "D": [2, 7, 8]}
    S = refrun.RefSession()
    arrays = {}
    for n, bonds in specs.items():
        arrays[n] = rng.uniform(-1, 1, wl.elem_count(bonds))
        S.tensor(n, bonds, labels[n], arrays[n])
    S.network("R", GREEDY_NET, {n: n for n in specs})
    S.save("R")
    o = S.run()
    arrays["R"] = o["R"]["elem"]
    w.add({"id": "greedy_net", "kind": "network", "net": GREEDY_NET,
           "tensors": {n: tensor_meta(specs[n], labels[n]) for n in specs}, "R": out_meta(o["R"])}, arrays)


def eigh_cases(w: Writer, rng):
    """Block::eigh (dsyev) of every block of square-block U(1) tensors, one
    IN and one OUT bond with equal charges and degeneracies; the inputs are
    not symmetric, so the fixture also pins which triangle dsyev reads."""
    specs = [[(-2, 1), (-1, 4), (0, 9), (1, 30), (2, 2)], [(0, 64)], [(-1, 3), (1, 3)]]
    for i, runs in enumerate(specs):
        bonds = [(1, [(u, 0, 0, d) for u, d in runs]), (-1, [(u, 0, 0, d) for u, d in runs])]
        n = sum(d * d for _, d in runs)
        elem = rng.standard_normal(n)
        if i == 2:  # symmetric blocks with a repeated eigenvalue
            elem = np.concatenate([np.eye(3).ravel() * 2.0, np.diag([1.0, 1.0, -1.0]).ravel()])
        S = refrun.RefSession()
        S.tensor("T", bonds, [1, 2], elem)
        for j, (u, _) in enumerate(runs):
            S.eigh("T", (u, 0, 0), f"e{j}")
        o = S.run()
        arrays = {"elem": elem}
        for j in range(len(runs)):
            e, v = o[f"e{j}"]
            arrays[f"E{j}"] = np.atleast_1d(np.asarray(e)).ravel()
            arrays[f"V{j}"] = np.atleast_2d(v)
        w.add({"id": f"eigh{i}", "kind": "eigh", "bonds": [[t, [list(r) for r in rr]] for t, rr in bonds],
               "blocks": [[u, d] for u, d in runs]}, arrays)


FNETS = [
    # (net text, [(name, [(label, type)])]): a label's second tensor gets Bond::change of the first's bond
    ("A: 1 2; 3\nB: 3 4; 5\nC: 5 1; 6\nTOUT: 2 4; 6\nORDER: ((B C) A)\n",
     [("A", [(1, 1), (2, 1), (3, -1)]), ("B", [(3, 1), (4, 1), (5, -1)]), ("C", [(5, 1), (1, 1), (6, -1)])]),
    ("A: 1 2; 3\nB: 3 4; 5\nC: 5 1; 6\nTOUT: 2 4; 6\n",
     [("A", [(1, 1), (2, 1), (3, -1)]), ("B", [(3, 1), (4, 1), (5, -1)]), ("C", [(5, 1), (1, 1), (6, -1)])]),
    ("A: 1; 2 3\nB: 2 4; 5\nC: 3 5; 6\nD: 6; 1 7\nTOUT: 4; 7\nORDER: ((C D) (B A))\n",
     [("A", [(1, 1), (2, -1), (3, -1)]), ("B", [(2, 1), (4, 1), (5, -1)]), ("C", [(3, 1), (5, 1), (6, -1)]),
      ("D", [(6, 1), (1, -1), (7, -1)])]),
]


def fermion_gates(w: Writer, rng, ngate: int, nnet: int):
    """UniTensor::addGate on random fermionic tensors, and fermionic networks
    whose contraction order differs from the file order, so Network::launch
    puts swap gates (addSwap, Network.cpp:944-993) on the tensors."""
    made = 0
    while made < ngate:
        rank = int(rng.integers(2, 6))
        bonds = rand_tensor(rng, rank, "fermion")
        if all(len(runs) == 1 for _, runs in bonds):
            continue
        pairs = []
        for _ in range(int(rng.integers(1, 5))):
            b1, b2 = (int(v) for v in rng.choice(rank, size=2, replace=False))
            pairs.append((b1, b2))
        labels = list(range(10, 10 + rank))
        el = rng.uniform(-1, 1, wl.elem_count(bonds))
        S = refrun.RefSession()
        S.tensor("T", bonds, labels, el)
        S.cmd("addgate T " + " ".join(f"{a} {b}" for a, b in pairs))
        S.save("T", "G")
        o = S.run()
        w.add({"id": f"fgate{made}", "kind": "addgate", "T": tensor_meta(bonds, labels), "swaps": pairs,
               "out": out_meta(o["G"])}, {"T": el, "G": o["G"]["elem"]})
        made += 1
    made = 0
    tries = 0
    while made < nnet:
        tries += 1
        net, spec = FNETS[made % len(FNETS)]
        first = {}
        tens = []
        for name, legs in spec:
            bonds = []
            for lab, t in legs:
                if lab not in first:
                    first[lab] = rand_bond(rng, t, "fermion_rich")
                    bonds.append(first[lab])
                else:
                    bonds.append(wl.change(first[lab], t))
            tens.append((name, bonds, [lab for lab, _ in legs]))
        if any(wl.elem_count(b) == 0 for _, b, _ in tens):
            continue
        S = refrun.RefSession()
        els = {}
        for name, bonds, labels in tens:
            els[name] = rng.uniform(-1, 1, wl.elem_count(bonds))
            S.tensor(name, bonds, labels, els[name])
        S.network("R", net, {name: name for name, _, _ in tens})
        S.save("R")
        try:
            o = S.run()
        except RuntimeError:
            continue
        if "R" not in o or o["R"]["elem"].size == 0 or not np.any(o["R"]["elem"]):
            continue  # no sector survives the contraction: the gates could not show
        w.add({"id": f"fnet{made}", "kind": "fnet", "net": net,
               "tensors": {name: tensor_meta(bonds, labels) for name, bonds, labels in tens}, "R": out_meta(o["R"])},
              {**els, "R": o["R"]["elem"]})
        made += 1


def legacy(refroot: str):
    ex = os.path.join(refroot, "Swig", "examples")
    out = {}
    meta = {}
    for f in ("egU3_W", "egU3_WT", "egU1_H_U1"):
        path = os.path.join(ex, f)
        d = uni10_io.read_legacy(path)
        with open(path, "rb") as fh:
            raw = fh.read()
        if uni10_io.legacy_bytes(d["bonds"], d["labels"], d["elem"], d["status"]) != raw:
            raise SystemExit(f"legacy writer does not reproduce {f}")
        out[f] = d["elem"]
        meta[f] = {"bonds": [[t, [list(r) for r in runs]] for t, runs in d["bonds"]], "labels": d["labels"],
                   "status": d["status"], "sha256": hashlib.sha256(raw).hexdigest()}
    for f in ("mat_U", "mat_Sigma", "mat_VT"):
        out[f] = np.fromfile(os.path.join(ex, f), dtype="<f8")
    out["_meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez(os.path.join(HERE, "legacy.npz"), **out)


# tensors saved by UniTensor::save: (file, bond signature, labels, name, with elements)
SAVED = [
    ("u1_rank3", [wl.u1_bond(1, (-1, 0, 1), (2, 3, 1)), wl.u1_bond(1, (1, -1), (1, 1)),
                  wl.u1_bond(-1, (-2, -1, 0, 1, 2), (1, 2, 3, 2, 1))], [4, -2, 7], "ALa", True),
    ("z2_fermion_rank4", [(1, [(0, 0, 0, 2), (0, 1, 1, 3)]), (1, [(0, 0, 0, 1), (0, 1, 1, 2)]),
                          (-1, [(0, 0, 0, 2), (0, 1, 1, 2)]), (-1, [(0, 1, 1, 1), (0, 0, 0, 3)])], [0, 1, 2, 3], "", True),
    ("dense_rank2", [wl.dense_bond(1, 5), wl.dense_bond(-1, 7)], [10, 11], "M", True),
    ("u1_no_elements", [wl.u1_bond(1, (0, 1), (2, 2)), wl.u1_bond(-1, (0, 1), (3, 1))], [0, 1], "empty", False),
]


def saved_files():
    """UniTensor::save of seeded tensors by the compiled reference."""
    d = os.path.join(HERE, "saved")
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(6006)
    index = []
    S = refrun.RefSession()
    for fname, bonds, labels, name, with_elem in SAVED:
        el = rng.uniform(-1, 1, wl.elem_count(bonds))
        if with_elem:
            S.tensor(fname, bonds, labels, el)
        else:
            S.lines.append(f"tensor {fname} {len(bonds)}")
            S.lines += [refrun.bond_line(b) for b in bonds]
            S.lines.append("labels " + fname + " " + " ".join(map(str, labels)))
        if name:
            S.cmd(f"name {fname} {name}")
        S.cmd(f"save {fname} {os.path.join(d, fname + '.uni10')}")
        index.append({"file": fname + ".uni10", "bonds": [[t, [list(r) for r in runs]] for t, runs in bonds],
                      "labels": labels, "name": name or fname,  # the driver names a tensor after its handle
                      "elem": [float(x) for x in el] if with_elem else None})
    S.run()
    with open(os.path.join(HERE, "saved.json"), "w") as f:
        json.dump(index, f, indent=0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--refroot", required=True, help="the reference project's uni10/ directory")
    ap.add_argument("--only", default="", help="comma-separated subset: saved, legacy")
    args = ap.parse_args()
    if not refrun.available():
        sys.exit("build oracle/_ref first: make -C oracle/refbuild")
    if args.only:
        parts = set(args.only.split(","))
        if "saved" in parts:
            saved_files()
        if "legacy" in parts:
            legacy(args.refroot)
        return
    rng = np.random.default_rng(12345)
    w = Writer()
    workload1(w)
    workload2(w)
    workload3_small(w)
    workload4_small(w)
    workload5_small(w)
    greedy_network(w, rng)
    permute_cases(w, rng, 40)
    contract_cases(w, rng, 30)
    # fermionic signs of permute / contract, with a stream of their own
    fermion_cases(w, np.random.default_rng(777), 16, 8)
    eigh_cases(w, np.random.default_rng(4242))
    fermion_gates(w, np.random.default_rng(909), 12, 15)
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(w.cases, f, indent=0)
    np.savez_compressed(os.path.join(HERE, "arrays.npz"), **w.arrays)
    legacy(args.refroot)
    print(f"{len(w.cases)} cases, {sum(a.size for a in w.arrays.values())} doubles")


if __name__ == "__main__":
    main()
