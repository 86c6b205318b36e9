"""Readers/writers for the reference's binary UniTensor layouts -- TEST ORACLE.

Current layout (UniTensor::save, tensor-network/lib/UniTensor.cpp:922-986;
reader :486-583):
    int r_flag; int c_flag; int namelen; char name[namelen]; int status;
    int bondNum; size_t sizeof(Qnum)=12;
    per bond { int type; int num_q; Qnum[num_q] (int U1, int prt, int prtF);
               int Qdegs[num_q] }
    int num_l; int labels[num_l]; [size_t elemNum; double elem[elemNum]]
Legacy layout (the reference's fixtures Swig/examples/egU1_H_U1, egU3_W,
egU3_WT): the same without the r_flag, c_flag, namelen, name prefix.
The elements are present when status has HAVEELEM (bit 2).
"""
from __future__ import annotations

import struct

import numpy as np

HAVEBOND, HAVEELEM = 1, 2


def _read_body(buf: bytes, pos: int):
    (status,) = struct.unpack_from("<i", buf, pos)
    pos += 4
    (bond_num,) = struct.unpack_from("<i", buf, pos)
    pos += 4
    (qsz,) = struct.unpack_from("<Q", buf, pos)
    pos += 8
    if qsz != 12:
        raise ValueError("unexpected sizeof(Qnum)")
    bonds = []
    for _ in range(bond_num):
        btype, nq = struct.unpack_from("<ii", buf, pos)
        pos += 8
        qn = np.frombuffer(buf, dtype="<i4", count=3 * nq, offset=pos).reshape(nq, 3)
        pos += 12 * nq
        deg = np.frombuffer(buf, dtype="<i4", count=nq, offset=pos)
        pos += 4 * nq
        bonds.append((int(btype), [(int(q[0]), int(q[1]), int(q[2]), int(d)) for q, d in zip(qn, deg)]))
    (nl,) = struct.unpack_from("<i", buf, pos)
    pos += 4
    labels = [int(x) for x in np.frombuffer(buf, dtype="<i4", count=nl, offset=pos)]
    pos += 4 * nl
    elem = None
    if status & HAVEELEM:
        (n,) = struct.unpack_from("<Q", buf, pos)
        pos += 8
        elem = np.frombuffer(buf, dtype="<f8", count=n, offset=pos).copy()
        pos += 8 * n
    return {"status": status, "bonds": bonds, "labels": labels, "elem": elem}, pos


def read_tensor(path: str) -> dict:
    with open(path, "rb") as f:
        buf = f.read()
    rflag, cflag, namelen = struct.unpack_from("<iii", buf, 0)
    name = buf[12 : 12 + namelen].decode("latin-1")
    d, _ = _read_body(buf, 12 + namelen)
    d.update(rflag=rflag, cflag=cflag, name=name)
    return d


def read_legacy(path: str) -> dict:
    with open(path, "rb") as f:
        buf = f.read()
    d, _ = _read_body(buf, 0)
    return d


def write_tensor(path: str, bonds, labels, elem, name: str = "") -> None:
    """UniTensor::save layout for a real tensor (r_flag=RTYPE=1, c_flag=CNULL=0)."""
    out = bytearray()
    nb = name.encode("latin-1")
    out += struct.pack("<iii", 1, 0, len(nb)) + nb
    out += struct.pack("<iiQ", HAVEBOND | HAVEELEM, len(bonds), 12)
    for btype, runs in bonds:
        out += struct.pack("<ii", btype, len(runs))
        for (u, p, f, _) in runs:
            out += struct.pack("<iii", u, p, f)
        for (_, _, _, d) in runs:
            out += struct.pack("<i", d)
    out += struct.pack("<i", len(labels)) + struct.pack(f"<{len(labels)}i", *labels)
    e = np.ascontiguousarray(elem, dtype="<f8")
    out += struct.pack("<Q", e.size) + e.tobytes()
    with open(path, "wb") as f:
        f.write(out)


def legacy_bytes(bonds, labels, elem, status: int = HAVEBOND | HAVEELEM) -> bytes:
    """The older layout (no r_flag, c_flag, name): the bytes of the reference's
    own fixtures (Swig/examples/egU3_W ...)."""
    out = bytearray(struct.pack("<iiQ", status, len(bonds), 12))
    for btype, runs in bonds:
        out += struct.pack("<ii", btype, len(runs))
        for (u, p, f, _) in runs:
            out += struct.pack("<iii", u, p, f)
        for (_, _, _, d) in runs:
            out += struct.pack("<i", d)
    out += struct.pack("<i", len(labels)) + struct.pack(f"<{len(labels)}i", *labels)
    if status & HAVEELEM:
        e = np.ascontiguousarray(elem, dtype="<f8")
        out += struct.pack("<Q", e.size) + e.tobytes()
    return bytes(out)
