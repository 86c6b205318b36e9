"""CPU restatement of Uni10's symmetric block-tensor path -- TEST ORACLE ONLY.

This module is test infrastructure.  Only the tests, ``__graft_entry__.smoke``
and ``bench.py``'s CPU-baseline / reference arm may import it, and only as the
checker or the timed CPU baseline; the product (``trim_gb300``) never does.

It restates, in numpy, the algorithms of the reference (Uni10 v1.0.0) for:
  * Qnum fusion / order / negation  (uni10/src/uni10/datatype/lib/Qnum.cpp:62-100)
  * Bond run-length setting, change, combine
                                    (data-structure/lib/Bond.cpp:90-110, 150-157, 163-237)
  * UniTensor::grouping (sector map) (tensor-network/lib/UniTensorReal.cpp:1169-1321)
  * initBlocks (block layout)        (UniTensorReal.cpp:1365-1374)
  * UniTensor::permute               (UniTensorReal.cpp:532-768)
  * UniTensor::transpose             (UniTensorReal.cpp:448-506)
  * UniTensor::combineBond           (UniTensorReal.cpp:791-866)
  * contract(rflag, Ta, Tb, fast)    (tensor-network/lib/UniTensorTools.cpp:124-244)
  * otimes                           (UniTensorTools.cpp:246-273)
  * Network fromfile/construct/launch/merge and the greedy planner
                                    (tensor-network/lib/Network.cpp:63-135, 271-506, 602-739)
  * fermionic swap gates: UniTensor::addGate (UniTensorReal.cpp:868-921),
    exSwap (UniTensor.cpp:1237-1268), recSwap (tools/lib/uni10_tools.cpp:44-69)
    and Network::addSwap / launch (Network.cpp:697-717, 923-993)
  * Block::svd via LAPACK dgesvd     (numeric/lapack/lib/uni10_lapack_cpu.cpp:289-313)
  * Block::eigh via LAPACK dsyev     (data-structure/lib/BlockReal.cpp:359-391,
                                     uni10_lapack_cpu.cpp:131-152)
  * the iTEBD truncation + normalisation over U(1) sectors
                                    (examples/iTEBD.cpp:153-171, Matrix::resize
                                     tensor-network/lib/MatrixReal.cpp:289-360)

Per-sector GEMMs call numpy's BLAS (``@``), as the reference calls dgemm_
(uni10_lapack_cpu.cpp:41-44).  The bit-exact parts (sector map, permute) are
pinned against the compiled reference (oracle/_ref) and against the
reference's own fixtures (Swig/examples/egU3_W, egU3_WT); see tests/golden.
Fermionic signs of permute (UniTensorReal.cpp:654-681, 733-738) are restated
and pinned by fermionic fixtures of the compiled reference; transpose carries
no sign (UniTensorReal.cpp:448-506), as in the reference.
"""
from __future__ import annotations

import bisect
import itertools
import re
from dataclasses import dataclass, field

import numpy as np

BD_IN = 1  # bondType values, uni10/src/uni10/data-structure/uni10_struct.h
BD_OUT = -1
PRT_EVEN, PRT_ODD = 0, 1
PRTF_EVEN, PRTF_ODD = 0, 1


# --------------------------------------------------------------------------- Qnum
@dataclass(frozen=True)
class Qnum:
    """Quantum number (U1, parity, fermionic parity); Qnum.h:52-170."""

    u1: int = 0
    prt: int = PRT_EVEN
    prtf: int = PRTF_EVEN

    def hash(self) -> int:  # Qnum.cpp:100 -- the order of blocks
        return self.u1 * 4 + self.prt * 2 + self.prtf

    def __mul__(self, o: "Qnum") -> "Qnum":  # Qnum.cpp:76-79 -- fusion
        return Qnum(self.u1 + o.u1, self.prt ^ o.prt, self.prtf ^ o.prtf)

    def __neg__(self) -> "Qnum":  # Qnum.cpp:71-74
        return Qnum(-self.u1, self.prt, self.prtf)

    def __lt__(self, o: "Qnum") -> bool:  # Qnum.cpp:62-64
        return self.hash() < o.hash()


# --------------------------------------------------------------------------- Bond
class Bond:
    """Run-length (Qnums, Qdegs) bond; Bond.cpp:90-110."""

    def __init__(self, btype: int, qlist):
        if len(qlist) == 0:
            raise ValueError("Cannot create a bond of dimension 0.")
        self.type = btype
        self.qnums: list[Qnum] = []
        self.qdegs: list[int] = []
        for i, q in enumerate(qlist):
            if i == 0 or q != qlist[i - 1]:
                self.qnums.append(q)
                self.qdegs.append(1)
            else:
                self.qdegs[-1] += 1

    @classmethod
    def from_runs(cls, btype: int, runs):
        """runs: [(Qnum, deg), ...]; equivalent to the reference's Qlist form."""
        qlist = [q for q, d in runs for _ in range(d)]
        return cls(btype, qlist)

    def copy(self) -> "Bond":
        b = Bond.__new__(Bond)
        b.type, b.qnums, b.qdegs = self.type, list(self.qnums), list(self.qdegs)
        return b

    def dim(self) -> int:
        return sum(self.qdegs)

    def change(self, tp: int) -> "Bond":  # Bond.cpp:150-157 -- flips and negates
        if self.type != tp:
            self.qnums = [-q for q in self.qnums]
            self.type = tp
        return self

    def combine(self, bd: "Bond") -> "Bond":  # Bond.cpp:163-197
        bd = bd.copy().change(self.type)
        qn: list[Qnum] = []
        qd: list[int] = []
        for q, d in zip(self.qnums, self.qdegs):
            for _ in range(d):
                for qq, dd in zip(bd.qnums, bd.qdegs):
                    f = q * qq
                    if not qn or f != qn[-1]:
                        qn.append(f)
                        qd.append(dd)
                    else:
                        qd[-1] += dd
        self.qnums, self.qdegs = qn, qd
        return self

    def __eq__(self, o) -> bool:  # Bond.cpp:147-149
        return self.type == o.type and self.qnums == o.qnums and self.qdegs == o.qdegs

    def __repr__(self) -> str:
        return f"Bond({'IN' if self.type == BD_IN else 'OUT'}, {[(q.u1, q.prt, q.prtf, d) for q, d in zip(self.qnums, self.qdegs)]})"


def combine_bonds(tp: int, bds: list[Bond]) -> Bond:
    """combine(bondType, vector<Bond>) -- Bond.cpp:198-238 (right-to-left fold)."""
    if not bds:
        raise ValueError("There should be at least one bond in the input vector to be combined.")
    if len(bds) == 1:
        return bds[0].copy().change(tp)
    n = len(bds)
    out1 = bds[n - 1].copy()
    out2 = bds[n - 2].copy()
    out2.change(tp)
    out2.combine(out1)
    b = 0
    while b < n - 2:
        if b % 2 == 0:
            out1 = bds[n - 3 - b].copy()
            out1.change(tp)
            out1.combine(out2)
        else:
            out2 = bds[n - 3 - b].copy()
            out2.change(tp)
            out2.combine(out1)
        b += 1
    return out2 if b % 2 == 0 else out1


# --------------------------------------------------------------------------- grouping
@dataclass
class SectorMap:
    """Result of UniTensor::grouping (UniTensorReal.cpp:1169-1321) + initBlocks."""

    rbond_num: int
    rqdim: int
    cqdim: int
    blocks: list = field(default_factory=list)  # [(Qnum, rows, cols, offset)] in Qnum order
    block_index: dict = field(default_factory=dict)  # Qnum -> index in blocks
    rq2blk: dict = field(default_factory=dict)  # row Qidx -> block index
    rq2off: dict = field(default_factory=dict)
    rq2dim: dict = field(default_factory=dict)
    cq2off: dict = field(default_factory=dict)
    cq2dim: dict = field(default_factory=dict)
    qidx_enc: list = field(default_factory=list)  # sorted Qidx keys (QidxEnc map order)
    elem_num: int = 0


def _odometer(bonds):
    """Odometer over Qnum indices, last bond fastest (UniTensorReal.cpp:1225-1233)."""
    return itertools.product(*[range(len(b.qnums)) for b in bonds])


def grouping(bonds: list[Bond]) -> SectorMap:
    rbn = 0
    in_before_out = True
    rqdim = cqdim = 1
    for b in bonds:
        if b.type == BD_IN:
            if not in_before_out:
                raise ValueError("Error in the input bond array: BD_OUT bonds must be placed after all BD_IN bonds.")
            rqdim *= len(b.qnums)
            rbn += 1
        else:
            cqdim *= len(b.qnums)
            in_before_out = False
    rows, cols = bonds[:rbn], bonds[rbn:]
    row_mdim: dict[Qnum, int] = {}
    row_q2idx: dict[Qnum, list[int]] = {}
    t_r_off, t_r_dim = {}, {}
    if rows:
        for boff, idxs in enumerate(_odometer(rows)):
            q, dim = Qnum(), 1
            for b, i in zip(rows, idxs):
                q = q * b.qnums[i]
                dim *= b.qdegs[i]
            t_r_off[boff] = row_mdim.get(q, 0)
            t_r_dim[boff] = dim
            row_mdim[q] = row_mdim.get(q, 0) + dim
            row_q2idx.setdefault(q, []).append(boff)
    else:
        row_mdim[Qnum()] = 1
        row_q2idx[Qnum()] = [0]
        t_r_off[0], t_r_dim[0] = 0, 1
    col_mdim: dict[Qnum, int] = {}
    col_q2idx: dict[Qnum, list[int]] = {}
    t_c_off, t_c_dim = {}, {}
    if cols:
        for boff, idxs in enumerate(_odometer(cols)):
            q, dim = Qnum(), 1
            for b, i in zip(cols, idxs):
                q = q * b.qnums[i]
                dim *= b.qdegs[i]
            if q in row_mdim:
                t_c_off[boff] = col_mdim.get(q, 0)
                t_c_dim[boff] = dim
                col_mdim[q] = col_mdim.get(q, 0) + dim
                col_q2idx.setdefault(q, []).append(boff)
    else:
        if Qnum() in row_mdim:
            col_mdim[Qnum()] = 1
            col_q2idx[Qnum()] = [0]
            t_c_off[0], t_c_dim[0] = 0, 1
    sm = SectorMap(rbond_num=rbn, rqdim=rqdim, cqdim=cqdim)
    off = 0
    qidx = set()
    for q in sorted(col_mdim, key=Qnum.hash):  # std::map<Qnum,...> order
        r, c = row_mdim[q], col_mdim[q]
        bi = len(sm.blocks)
        sm.blocks.append((q, r, c, off))
        sm.block_index[q] = bi
        off += r * c
        for ri in row_q2idx[q]:
            sm.rq2blk[ri] = bi
            sm.rq2dim[ri] = t_r_dim[ri]
            sm.rq2off[ri] = t_r_off[ri]
            for ci in col_q2idx[q]:
                sm.cq2dim[ci] = t_c_dim[ci]
                sm.cq2off[ci] = t_c_off[ci]
                qidx.add(ri * cqdim + ci)
    sm.qidx_enc = sorted(qidx)
    sm.elem_num = off
    return sm


# --------------------------------------------------------------------------- UniTensor
class UniTensor:
    """Real (FP64) symmetric tensor: bonds, labels and the contiguous elem
    buffer whose blocks lie back to back in Qnum order, each row-major
    (UniTensorReal.cpp:1365-1374).

    ``diag`` marks a tensor with one row and one column bond whose blocks were
    all put as diagonal matrices (the reference's Lambda / singular-value
    matrices); contract() then applies it as a row or column scale, the
    diagonal paths of RDotR (BlockTools.cpp:45-60)."""

    diag = False

    def __init__(self, bonds: list[Bond], labels=None, elem=None, name: str = ""):
        self.bonds = [b.copy() for b in bonds]
        self.name = name
        if bonds:
            self.smap = grouping(self.bonds)
            if not self.smap.blocks:
                raise ValueError("There is no symmetry block with the given bonds")
            self.labels = list(range(len(bonds))) if labels is None else list(labels)
            n = self.smap.elem_num
        else:  # scalar tensor, UniTensorReal.cpp:1342-1350
            self.smap = None
            self.labels = []
            n = 1
        self.elem = np.zeros(n) if elem is None else np.array(elem, dtype=np.float64, copy=True)
        if self.elem.size != n:
            raise ValueError(f"element count {self.elem.size} != {n}")

    # -- accessors mirroring the reference API
    def elem_num(self) -> int:
        return self.elem.size

    def in_bond_num(self) -> int:
        return self.smap.rbond_num if self.smap else 0

    def block_qnums(self):
        return [b[0] for b in self.smap.blocks]

    def get_block(self, q: Qnum) -> np.ndarray:
        _, r, c, off = self.smap.blocks[self.smap.block_index[q]]
        return self.elem[off : off + r * c].reshape(r, c)

    def put_block(self, q: Qnum, mat, diag: bool = False, fresh: bool = False) -> None:
        """putBlock (UniTensorReal.cpp:208-239); with diag, ``mat`` is the
        diagonal and the rest of the block is zeroed.  ``fresh``: no element
        has been set since creation, so all-diagonal puts make a diagonal
        tensor."""
        blk = self.get_block(q)
        if diag:
            blk[...] = 0.0
            n = min(blk.shape)
            blk[np.arange(n), np.arange(n)] = np.asarray(mat, dtype=np.float64)[:n]
            if fresh or self.diag:
                self.diag = len(self.bonds) == 2 and self.in_bond_num() == 1
        else:
            blk[...] = mat
            self.diag = False

    def copy(self) -> "UniTensor":
        t = UniTensor.__new__(UniTensor)
        t.bonds = [b.copy() for b in self.bonds]
        t.name, t.smap, t.labels, t.elem = self.name, self.smap, list(self.labels), self.elem.copy()
        t.diag = self.diag
        return t

    def set_label(self, labels) -> None:
        if len(labels) != len(self.bonds):
            raise ValueError("The size of input vector(labels) does not match for the number of bonds.")
        self.labels = list(labels)

    # -- permute: UniTensorReal.cpp:532-768
    def permute(self, new_labels, row_bond_num: int) -> "UniTensor":
        if not self.bonds:
            raise ValueError("There is no bond in the tensor(scalar) to permute.")
        if len(new_labels) != len(self.labels):
            raise ValueError("The size of the input new labels does not match for the number of bonds.")
        n = len(self.bonds)
        rsp = [0] * n
        cnt = 0
        for i in range(n):
            for j in range(n):
                if self.labels[i] == new_labels[j]:
                    rsp[j] = i
                    cnt += 1
        if cnt != len(new_labels):
            raise ValueError("The input new labels do not 1-1 correspond to the labels of the tensor.")
        inorder = all(rsp[i] == i for i in range(1, n))
        if inorder and self.smap.rbond_num == row_bond_num:
            return self
        out_bonds = [self.bonds[rsp[b]].copy() for b in range(n)]
        for b in range(n):
            out_bonds[b].change(BD_IN if b < row_bond_num else BD_OUT)
        out = UniTensor(out_bonds, labels=list(new_labels), name=self.name)
        permute_elems(self, out, rsp)
        self.bonds, self.smap, self.labels, self.elem = out.bonds, out.smap, out.labels, out.elem
        self.diag = self.diag and n == 2 and row_bond_num == 1  # a block-wise transpose
        return self

    def permute_rows(self, row_bond_num: int) -> "UniTensor":  # UniTensorReal.cpp:508-518
        return self.permute(list(self.labels), row_bond_num)

    # -- transpose: UniTensorReal.cpp:448-506
    def transpose(self) -> "UniTensor":
        n = len(self.bonds)
        rbn = 0
        for b in self.bonds:
            if b.type == BD_IN:
                rbn += 1
            else:
                break
        cbn = n - rbn
        rsp = [rbn + b if b < cbn else b - cbn for b in range(n)]
        out_bonds = [self.bonds[rsp[b]].copy() for b in range(n)]
        for b in range(n):
            out_bonds[b].type = BD_IN if b < cbn else BD_OUT  # type set without negation
        out = UniTensor(out_bonds, labels=[self.labels[rsp[b]] for b in range(n)], name=self.name)
        for q, r, c, off in self.smap.blocks:
            out.put_block(q, self.elem[off : off + r * c].reshape(r, c).T)
        self.bonds, self.smap, self.labels, self.elem = out.bonds, out.smap, out.labels, out.elem
        return self

    # -- combineBond: UniTensorReal.cpp:791-866
    def combine_bond(self, cmb_labels) -> "UniTensor":
        if len(cmb_labels) < 2:
            return self
        picked = []
        marked = [0] * len(self.labels)
        for lab in cmb_labels:
            for li, l in enumerate(self.labels):
                if lab == l:
                    picked.append(li)
                    marked[li] = 1
                    break
        if sum(marked) != len(cmb_labels):
            raise ValueError("The input labels do not match for the labels of the tensor.")
        rsp, reduced, new_bonds, rbn = [], [], [], 0
        for li, l in enumerate(self.labels):
            if marked[li] and li == picked[0]:
                rsp.extend(cmb_labels)
                tmp = [self.bonds[p] for p in picked]
                if self.bonds[picked[0]].type == BD_IN:
                    rbn += len(picked)
                new_bonds.append(combine_bonds(tmp[0].type, tmp))
                reduced.append(l)
            elif not marked[li]:
                rsp.append(l)
                reduced.append(l)
                if self.bonds[li].type == BD_IN:
                    rbn += 1
                new_bonds.append(self.bonds[li].copy())
        self.permute(rsp, rbn)
        out = UniTensor(new_bonds, labels=reduced, elem=self.elem, name=self.name)
        self.bonds, self.smap, self.labels, self.elem = out.bonds, out.smap, out.labels, out.elem
        return self


def _subblock_dims(t: UniTensor, qidx: int):
    """Decode a Qidx into per-bond Qnum indices (UniTensorReal.cpp:705-712)."""
    idxs = [0] * len(t.bonds)
    tmp = qidx
    for b in range(len(t.bonds) - 1, -1, -1):
        qd = len(t.bonds[b].qnums)
        idxs[b] = tmp % qd
        tmp //= qd
    return idxs


def fermion_swaps(n: int, rbn_in: int, rbn_out: int, rsp):
    """Bond swaps that carry fermionic signs (UniTensorReal.cpp:656-681;
    recSwap, tools/lib/uni10_tools.cpp:48-67): in- and output bonds are put in
    the order row bonds, then column bonds reversed; the adjacent exchanges
    of a bubble sort of the output order (by input position) are the swaps,
    each named by its two input bonds."""
    ordf = [b if b < rbn_in else n - b + rbn_in - 1 for b in range(n)]  # bond -> position (an involution)
    ord_ = [0] * n
    for j in range(n):
        pj = j if j < rbn_out else n - j + rbn_out - 1
        ord_[pj] = ordf[rsp[j]]
    swaps = []
    for i in range(n - 1):
        for j in range(n - i - 1):
            if ord_[j] > ord_[j + 1]:
                swaps.append((ordf[ord_[j + 1]], ordf[ord_[j]]))
                ord_[j], ord_[j + 1] = ord_[j + 1], ord_[j]
    return swaps


def permute_elems(src: UniTensor, dst: UniTensor, rsp) -> None:
    """The data movement of permute: for every sub-block (Qidx in QidxEnc
    order) copy the input sub-block, viewed as a dense tensor over its bonds'
    degeneracies, into the output sub-block with bonds reordered by rsp
    (UniTensorReal.cpp:685-757).  Exact: pure data movement, times the
    sub-block's fermionic sign on the symmetric path (:653-681, 733-738)."""
    n = len(src.bonds)
    sm, dm = src.smap, dst.smap
    # the symmetric path: some input bond has more than one charge
    # (UniTensorReal.cpp:567-571); bosonic charges give +1 everywhere
    symmetric = any(len(b.qnums) != 1 for b in src.bonds)
    swaps = fermion_swaps(n, sm.rbond_num, dm.rbond_num, rsp) if symmetric else []
    qot_acc = [1] * n
    for b in range(n - 1, 0, -1):
        qot_acc[b - 1] = qot_acc[b] * len(dst.bonds[b].qnums)
    for qin in sm.qidx_enc:
        qi = _subblock_dims(src, qin)
        degs = [src.bonds[b].qdegs[qi[b]] for b in range(n)]
        qot = sum(qi[rsp[b]] * qot_acc[b] for b in range(n))
        rin, cin = divmod(qin, sm.cqdim)
        rot, cot = divmod(qot, dm.cqdim)
        _, _, bin_c, bin_off = sm.blocks[sm.rq2blk[rin]]
        _, _, bot_c, bot_off = dm.blocks[dm.rq2blk[rot]]
        srd, scd = sm.rq2dim[rin], sm.cq2dim[cin]
        ord_, ocd = dm.rq2dim[rot], dm.cq2dim[cot]
        s0 = bin_off + sm.rq2off[rin] * bin_c + sm.cq2off[cin]
        d0 = bot_off + dm.rq2off[rot] * bot_c + dm.cq2off[cot]
        sub = np.lib.stride_tricks.as_strided(
            src.elem[s0:], shape=(srd, scd), strides=(bin_c * 8, 8)
        )
        sub = sub.reshape(degs).transpose(rsp).reshape(ord_, ocd)
        parity = 0
        for b1, b2 in swaps:
            parity ^= src.bonds[b1].qnums[qi[b1]].prtf & src.bonds[b2].qnums[qi[b2]].prtf
        dview = np.lib.stride_tricks.as_strided(dst.elem[d0:], shape=(ord_, ocd), strides=(bot_c * 8, 8))
        dview[...] = -sub if parity else sub


# --------------------------------------------------------------------------- swap gates
def add_gate(t: UniTensor, swaps) -> None:
    """UniTensor::addGate (UniTensorReal.cpp:868-921): the sign of a sub-block
    is the XOR over the swaps (b1, b2) of prtF(b1's charge) & prtF(b2's
    charge); sub-blocks of sign -1 are negated in place."""
    if not t.bonds:
        raise ValueError("Adding swap gates to a tensor without bonds(scalar).")
    sm = t.smap
    for qin in sm.qidx_enc:
        qi = _subblock_dims(t, qin)
        parity = 0
        for b1, b2 in swaps:
            parity ^= t.bonds[b1].qnums[qi[b1]].prtf & t.bonds[b2].qnums[qi[b2]].prtf
        if parity:
            rin, cin = divmod(qin, sm.cqdim)
            _, _, bc, boff = sm.blocks[sm.rq2blk[rin]]
            s0 = boff + sm.rq2off[rin] * bc + sm.cq2off[cin]
            v = np.lib.stride_tricks.as_strided(t.elem[s0:], shape=(sm.rq2dim[rin], sm.cq2dim[cin]), strides=(bc * 8, 8))
            v[...] = -v


def ex_swap(ta: UniTensor, tb: UniTensor):
    """UniTensor::exSwap (UniTensor.cpp:1237-1268): (bond of ta whose label is
    in tb, bond of ta whose label is not) for every such pair."""
    inter = [a for a, l in enumerate(ta.labels) if l in tb.labels]
    left = [a for a, l in enumerate(ta.labels) if l not in tb.labels]
    return [(i, j) for i in inter for j in left]


def rec_swap(order):
    """recSwap(ord) (tools/lib/uni10_tools.cpp:44-69, ordF = identity): the
    adjacent exchanges of a bubble sort of ord, as (smaller, larger) values."""
    ord_ = list(order)
    out = []
    n = len(ord_)
    for i in range(n - 1):
        for j in range(n - i - 1):
            if ord_[j] > ord_[j + 1]:
                out.append((ord_[j + 1], ord_[j]))
                ord_[j], ord_[j + 1] = ord_[j + 1], ord_[j]
    return out


def network_swaps(root, tensors):
    """Network::addSwap (Network.cpp:923-993): the contraction order of the
    leaves (pre-order walk of the tree), its bubble-sort exchanges, each
    giving exSwap(T_b1, T_b2) to tensor b1; per tensor the pairs are kept when
    they occur an odd number of times, ordered by min * bondNum + max."""
    con = []

    def walk(nd):
        if nd is None or len(con) == len(tensors):
            return
        if nd.t is not None:
            con.append(nd.t)
        walk(nd.left)
        walk(nd.right)

    walk(root)
    arr = [[] for _ in tensors]
    for b1, b2 in rec_swap(con):
        arr[b1] += ex_swap(tensors[b1], tensors[b2])
    out = []
    for t, sw in zip(tensors, arr):
        nb = len(t.bonds)
        recs = {}
        for a, b in sw:
            h = min(a, b) * nb + max(a, b)
            recs[h] = not recs.get(h, False)
        out.append([(h // nb, h % nb) for h in sorted(recs) if recs[h]])
    return out


def is_fermionic(tensors) -> bool:
    """Whether any bond carries an odd fermionic parity (the reference keys
    the swap gates on Qnum::isFermionic, set by any PRTF_ODD charge; without
    one every gate sign is +1)."""
    return any(q.prtf for t in tensors for b in t.bonds for q in b.qnums)


# --------------------------------------------------------------------------- contract
def contract(ta: UniTensor, tb: UniTensor, fast: bool = False, gemm=None) -> UniTensor:
    """contract(rflag, Ta, Tb, fast) -- UniTensorTools.cpp:124-244.

    Mutates ``ta``/``tb`` (permutes them in place) and restores them when
    ``fast`` is false.  ``gemm(A, B)`` defaults to numpy's BLAS product."""
    if gemm is None:
        gemm = np.matmul
    if ta is tb:
        tb = tb.copy()
    if not ta.bonds or not tb.bonds:
        if ta.bonds:
            r = ta.copy(); r.elem *= tb.elem[0]; return r
        if tb.bonds:
            r = tb.copy(); r.elem *= ta.elem[0]; return r
        return UniTensor([], elem=ta.elem * tb.elem)
    an, bn = len(ta.bonds), len(tb.bonds)
    old_la, old_lb = list(ta.labels), list(tb.labels)
    old_ra, old_rb = ta.in_bond_num(), tb.in_bond_num()
    new_la, inter, new_lb, new_lc = [], [], [], []
    mark_b = [0] * bn
    for a in range(an):
        match = False
        for b in range(bn):
            if ta.labels[a] == tb.labels[b]:
                mark_b[b] = 1
                inter.append(ta.labels[a])
                new_lb.append(tb.labels[b])
                if ta.bonds[a].dim() != tb.bonds[b].dim():
                    raise ValueError("Cannot contract two bonds having different dimensions")
                match = True
                break
        if not match:
            new_la.append(ta.labels[a])
            new_lc.append(ta.labels[a])
    new_la += inter
    for b in range(bn):
        if not mark_b[b]:
            new_lb.append(tb.labels[b])
            new_lc.append(tb.labels[b])
    con = len(inter)
    ta.permute(new_la, an - con)
    tb.permute(new_lb, con)
    c_bonds = [ta.bonds[i] for i in range(an - con)] + [tb.bonds[i] for i in range(con, bn)]
    tc = UniTensor(c_bonds)
    if c_bonds:
        tc.set_label(new_lc)
    # a diagonal operand contracted over one bond: RDotR's diagRowMul /
    # diagColMul (BlockTools.cpp:45-60), no GEMM; rows (columns) beyond the
    # diagonal's length are zero, as the reference's resize leaves them
    da = ta.diag and an == 2 and con == 1
    db = not da and tb.diag and bn == 2 and con == 1
    for q, r, k, off in ta.smap.blocks:
        if q in tb.smap.block_index:
            bb = tb.get_block(q)
            cb = tc.get_block(q)
            if not (r == cb.shape[0] and bb.shape[1] == cb.shape[1] and k == bb.shape[0]):
                raise ValueError("The dimensions the bonds to be contracted out are different.")
            ab = ta.elem[off : off + r * k].reshape(r, k)
            if da:
                n = min(r, k)
                cb[:n] = np.diagonal(ab)[:n, None] * bb[:n]
                cb[n:] = 0.0
            elif db:
                n = min(bb.shape)
                cb[:, :n] = ab[:, :n] * np.diagonal(bb)[None, :n]
                cb[:, n:] = 0.0
            else:
                cb[...] = gemm(ab, bb)
    if con == 0:  # outer product, UniTensorTools.cpp:206-225
        lc = old_la[:old_ra] + old_lb[:old_rb] + old_la[old_ra:] + old_lb[old_rb:]
        tc.permute(lc, old_ra + old_rb)
    if not fast:
        ta.permute(old_la, old_ra)
        tb.permute(old_lb, old_rb)
    return tc


def otimes(ta: UniTensor, tb: UniTensor) -> UniTensor:  # UniTensorTools.cpp:246-273
    t1, t2 = ta.copy(), tb.copy()
    l1 = [i if i < t1.in_bond_num() else t2.in_bond_num() + i for i in range(len(t1.bonds))]
    l2 = [i + t1.in_bond_num() if i < t2.in_bond_num() else i + len(t1.bonds) for i in range(len(t2.bonds))]
    t1.set_label(l1)
    t2.set_label(l2)
    return contract(t1, t2, True)


def sector_gemms(ta: UniTensor, tb: UniTensor):
    """(M, N, K) of every sector GEMM contract() would issue for these operands
    (after its permutes); used for the algorithmic flop count."""
    a, b = ta.copy(), tb.copy()
    shapes = []
    contract(a, b, True, gemm=lambda x, y: (shapes.append((x.shape[0], y.shape[1], x.shape[1])), x @ y)[1])
    return shapes


# --------------------------------------------------------------------------- Network
def _cal_elem_num(bonds) -> int:
    """Node::cal_elemNum -- Network.cpp:137-223 (element count of grouping)."""
    rbn = sum(1 for b in bonds if b.type == BD_IN)
    cbn = sum(1 for b in bonds if b.type == BD_OUT)
    rows, cols = bonds[:rbn], bonds[rbn : rbn + cbn]
    row_m: dict[Qnum, int] = {}
    if rows:
        for idxs in _odometer(rows):
            q, d = Qnum(), 1
            for b, i in zip(rows, idxs):
                q = q * b.qnums[i]
                d *= b.qdegs[i]
            row_m[q] = row_m.get(q, 0) + d
    else:
        row_m[Qnum()] = 1
    col_m: dict[Qnum, int] = {}
    if cols:
        for idxs in _odometer(cols):
            q, d = Qnum(), 1
            for b, i in zip(cols, idxs):
                q = q * b.qnums[i]
                d *= b.qdegs[i]
            if q in row_m:
                col_m[q] = col_m.get(q, 0) + d
    elif Qnum() in row_m:
        col_m[Qnum()] = 1
    return sum(row_m[q] * c for q, c in col_m.items())


class _Node:
    def __init__(self, bonds, labels, tensor_idx=None, elem_num=None):
        self.bonds, self.labels, self.t = bonds, labels, tensor_idx
        self.elem_num = _cal_elem_num(bonds) if elem_num is None else elem_num
        self.parent = self.left = self.right = None
        self.point = 0.0

    def _pair(self, nd):
        cb, lc, mark_b, con = [], [], [0] * len(nd.bonds), 0
        for a, la in enumerate(self.labels):
            m = False
            for b, lb in enumerate(nd.labels):
                if la == lb:
                    mark_b[b] = 1
                    m = True
                    con += 1
                    break
            if not m:
                lc.append(la)
                cb.append(self.bonds[a].copy())
        for b, lb in enumerate(nd.labels):
            if not mark_b[b]:
                lc.append(lb)
                cb.append(nd.bonds[b].copy())
        rbn = len(self.bonds) - con
        for a in range(rbn):
            cb[a].change(BD_IN)
        for a in range(len(nd.bonds) - con):
            cb[rbn + a].change(BD_OUT)
        return cb, lc, con

    def contract(self, nd) -> "_Node":  # Network.cpp:63-101
        cb, lc, _ = self._pair(nd)
        return _Node(cb, lc)

    def metric(self, nd) -> float:  # Network.cpp:103-135
        cb, _, con = self._pair(nd)
        if con == 0:
            return -1.0
        # float(elemNum + nd->elemNum) / newElemNum in single precision
        return float(np.float32(self.elem_num + nd.elem_num) / np.float32(_cal_elem_num(cb)))


class Network:
    """Network (Network.cpp): .net parsing, contraction-tree construction
    (explicit ORDER brackets or the greedy matching/branch planner) and
    launch = recursive merge + final permute to TOUT."""

    def __init__(self, fname: str | None = None, text: str | None = None):
        if text is None:
            with open(fname) as f:
                text = f.read()
        self.names, self.label_arr, self.rnums, self.order, self.brakets = [], [], [], [], []
        self._parse(text)
        self.tensors: list[UniTensor | None] = [None] * (len(self.names) - 1)
        self.swapflags = [False] * (len(self.names) - 1)
        self.swaps = None  # per tensor, from the first construct (Network::addSwap)

    def _parse(self, text: str) -> None:  # Network.cpp:271-427
        ord_names = []
        for line in text.split("\n")[:1000]:
            pos = line.find(":")
            if pos < 0:
                break
            name = line[:pos].strip()
            rest = line[pos + 1 :]
            if name == "ORDER":
                if "(" not in rest:
                    ord_names = [w for w in re.split(r"[ ,;]+", rest) if w]
                else:
                    # each delimiter run before a name contributes -(#')')
                    # then +(#'('); the run after the last name -(#')')
                    # (Network.cpp:316-357)
                    start = re.search(r"[ ,;*()]", rest)
                    prev_end = start.start() if start else len(rest)
                    for m in re.finditer(r"[^ ,;*()]+", rest):
                        if m.start() < prev_end:
                            continue
                        run = rest[prev_end : m.start()]
                        if run.count(")"):
                            self.brakets.append(-run.count(")"))
                        if run.count("("):
                            self.brakets.append(run.count("("))
                        ord_names.append(m.group(0))
                        self.brakets.append(0)
                        prev_end = m.end()
                    tail = rest[prev_end:]
                    if tail.count(")"):
                        self.brakets.append(-tail.count(")"))
                    if sum(self.brakets) != 0:
                        raise ValueError("There are imbalance brackets when specifying the contraction order.")
                break
            self.names.append(name)
            semi = rest.find(";")
            labs, rnum = [], -1
            for m in re.finditer(r"[0-9-]+", rest):
                if rnum == -1 and semi >= 0 and semi < m.start():
                    rnum = len(labs)
                labs.append(int(m.group(0)))
            self.label_arr.append(labs)
            self.rnums.append(len(labs) if rnum == -1 else rnum)
        if not self.names or self.names[-1] != "TOUT":
            raise ValueError("Missing TOUT tensor.")
        if len(self.names) <= 2:
            raise ValueError("There must be at least two tensors in a tensor network.")
        num_t = len(self.names) - 1
        if ord_names:
            if len(ord_names) != num_t:
                raise ValueError("Some tensors are missing in the contraction order.")
            self.order = [self.names.index(n) for n in ord_names]
        else:
            self.order = list(range(num_t))

    def put_tensor(self, name_or_idx, t: UniTensor) -> None:  # Network.cpp:508-541
        idx = self.names.index(name_or_idx) if isinstance(name_or_idx, str) else name_or_idx
        if t.in_bond_num() != self.rnums[idx]:
            raise ValueError("The number of in-coming bonds does not match with the tensor specified in network file")
        c = t.copy()
        c.set_label(self.label_arr[idx])
        c.name = self.names[idx]
        self.tensors[idx] = c
        self.swapflags[idx] = False  # Network.cpp:524-528

    # -- construct: Network.cpp:428-506 and the greedy planner :602-670
    def construct(self):
        leafs = [_Node([b.copy() for b in t.bonds], list(t.labels), i, t.elem_num()) for i, t in enumerate(self.tensors)]
        self.root = None
        if self.brakets:
            stack, cnt = [], 0
            for br in self.brakets:
                if br < 0:
                    for _ in range(-br):
                        par = stack[-2].contract(stack[-1])
                        par.left, par.right = stack[-2], stack[-1]
                        stack[-2:] = [par]
                        if len(stack) < 2:
                            break
                elif br == 0:
                    stack.append(leafs[self.order[cnt]])
                    cnt += 1
            while len(stack) > 1:
                par = stack[-2].contract(stack[-1])
                par.left, par.right = stack[-2], stack[-1]
                stack[-2:] = [par]
            self.root = stack[0]
        else:
            for i in self.order:
                self._matching(leafs[i], self.root)
        tout = self.label_arr[-1]
        if len(self.root.labels) != len(tout) or set(self.root.labels) != set(tout):
            raise ValueError("The labels of the resulting tensor do not match with the labels of 'TOUT'")
        return self.root

    def _branch(self, sbj, tar):  # Network.cpp:602-649
        par = tar.contract(sbj)
        if sbj.parent is None:
            if tar.parent is not None:
                if tar.parent.left is tar:
                    tar.parent.left = par
                else:
                    tar.parent.right = par
                par.parent = tar.parent
            else:
                par.parent = None
                self.root = par
        else:
            gp = tar.parent.parent
            if gp is not None:
                if gp.left is tar.parent:
                    gp.left = par
                else:
                    gp.right = par
                par.parent = gp
            else:
                par.parent = None
                self.root = par
        par.left, par.right = tar, sbj
        tar.parent = sbj.parent = par
        par.point = tar.metric(sbj)
        if sbj.parent.parent is not None:
            sbj = sbj.parent
            self._branch(sbj.parent.right, sbj.parent.left)

    def _matching(self, sbj, tar):  # Network.cpp:651-670
        if tar is None:
            self.root = sbj
        elif tar.t is None:
            if sbj.metric(tar) > 0:
                tar_p = tar.point
                lft_p = rht_p = 0.0
                lft_p = sbj.metric(tar.left)
                go = lft_p > tar_p
                if not go:
                    rht_p = sbj.metric(tar.right)
                    go = rht_p > tar_p
                if go:
                    self._matching(sbj, tar.left if lft_p > rht_p else tar.right)
                else:
                    self._branch(sbj, tar)
            else:
                self._branch(sbj, tar)
        else:
            self._branch(sbj, tar)

    def _merge(self, nd, gemm=None) -> UniTensor:  # Network.cpp:719-739
        l = self._merge(nd.left, gemm) if nd.left.t is None else self.tensors[nd.left.t]
        r = self._merge(nd.right, gemm) if nd.right.t is None else self.tensors[nd.right.t]
        return contract(l, r, True, gemm=gemm)

    def launch(self, gemm=None) -> UniTensor:  # Network.cpp:697-717
        root = self.construct()
        if self.swaps is None:
            self.swaps = network_swaps(root, self.tensors) if is_fermionic(self.tensors) else [[] for _ in self.tensors]
        for t, sw in enumerate(self.swaps):
            if not self.swapflags[t]:
                if sw:
                    add_gate(self.tensors[t], sw)
                self.swapflags[t] = True
        out = self._merge(root, gemm)
        tout = self.label_arr[-1]
        if len(tout) > 1:
            out.permute(tout, self.rnums[-1])
        return out

    def tree(self):
        """Contraction tree as nested tuples of tensor names (for comparison)."""
        def rec(nd):
            return self.names[nd.t] if nd.t is not None else (rec(nd.left), rec(nd.right))
        return rec(self.construct())


# --------------------------------------------------------------------------- SVD
def block_svd(mat: np.ndarray):
    """Block::svd -> (U, S, VT) via LAPACK dgesvd ('S','S'); uni10_lapack_cpu.cpp:289-313."""
    import scipy.linalg

    u, s, vt = scipy.linalg.svd(mat, full_matrices=False, lapack_driver="gesvd")
    return u, s, vt


def block_eigh(mat: np.ndarray):
    """Block::eigh -> (E, V) via LAPACK dsyev ('V', 'U'); BlockReal.cpp:359-391,
    uni10_lapack_cpu.cpp:131-152.

    The reference hands the row-major N x N buffer to the column-major dsyev,
    which reads its upper triangle: the LOWER triangle of the row-major matrix
    (row >= column).  E holds the eigenvalues in ascending order; dsyev leaves
    eigenvector j in column j of its column-major output, so in the row-major
    Matrix the reference returns, row j of V is eigenvector j."""
    import scipy.linalg

    a = np.asarray(mat, dtype=np.float64)
    n = a.shape[0]
    if a.ndim != 2 or a.shape[1] != n:
        raise ValueError("Cannot perform eigenvalue decomposition on a non-square matrix.")
    low = np.tril(a)
    sym = low + np.tril(a, -1).T
    e, v = scipy.linalg.eigh(sym, driver="ev")
    return e, np.ascontiguousarray(v.T)


# --------------------------------------------------------------------------- truncation
def truncate_global(svals, chi: int):
    """Keep the chi largest singular values over all sectors and normalise.

    The reference example keeps the leading chi of its single sector
    (examples/iTEBD.cpp:156-159: ``rets[1].resize(dim, dim).norm()`` then
    ``rets[1] *= (1 / norm)``); over U(1) sectors the leading chi are taken
    from the values of all sectors together, ordered by value descending,
    ties by lower sector index, then lower position.  Returns (kept counts,
    norm, normalised kept values per sector)."""
    entries = sorted((-float(v), q, i) for q, sv in enumerate(svals) for i, v in enumerate(sv))[: max(0, chi)]
    kept = [0] * len(svals)
    for _, q, _ in entries:
        kept[q] += 1
    allkept = np.concatenate([np.asarray(sv[:k], dtype=np.float64) for sv, k in zip(svals, kept)] or [np.zeros(0)])
    norm = float(np.linalg.norm(allkept))
    inv = 1.0 / norm if norm > 0 else float("inf")
    return kept, norm, [np.asarray(sv[:k], dtype=np.float64) * inv for sv, k in zip(svals, kept)]


def svd_truncate(theta: "UniTensor", chi: int):
    """Block SVD of theta (row bonds | column bonds), truncated to the chi
    largest singular values over all blocks and normalised: the U(1) form of
    the iTEBD update (examples/iTEBD.cpp:153-171).  Returns U [row bonds | n],
    S [n | n] (diagonal blocks), VT [n | column bonds] and the norm, where the
    new bond n carries charge q at the multiplicity kept in block q and the
    labels chain U . S . VT back to theta's labels."""
    qs = theta.block_qnums()
    svds = [block_svd(theta.get_block(q)) for q in qs]
    kept, norm, snorm = truncate_global([sv[1] for sv in svds], chi)
    ql = [q for q, k in zip(qs, kept) for _ in range(k)]
    nin, nout = Bond(BD_IN, ql), Bond(BD_OUT, ql)
    rb = theta.in_bond_num()
    nl = max(theta.labels) + 1 if theta.labels else 0
    U = UniTensor(theta.bonds[:rb] + [nout], labels=theta.labels[:rb] + [nl])
    S = UniTensor([nin, nout], labels=[nl, nl + 1])
    VT = UniTensor([nin] + theta.bonds[rb:], labels=[nl + 1] + theta.labels[rb:])
    for q, (u, _, vt), k, sn in zip(qs, svds, kept, snorm):
        if k == 0:
            continue
        U.put_block(q, u[:, :k])
        S.put_block(q, np.diag(sn))
        VT.put_block(q, vt[:k, :])
    return U, S, VT, norm
