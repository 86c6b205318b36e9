"""Python mirror of the reference's UniTensor / Network operations on this
path (the calls the reference's SWIG module, pyUni10, exposes), over the C
ABI.  Bonds use the run-length form ``(btype, [(u1, prt, prtf, deg), ...])``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import MODES, call, int_array, pack_bonds


def _mode(mode) -> int:
    return MODES[mode] if isinstance(mode, str) else int(mode)


class SectorMap:
    """Cached sector map of a bond signature (UniTensor::grouping)."""

    def __init__(self, bonds):
        self.bonds = bonds
        h = C.c_void_p()
        call("tn_sectormap_build", None, *pack_bonds(bonds), C.byref(h))
        self.h = h
        n, nb, rb = C.c_int64(), C.c_int(), C.c_int()
        call("tn_sectormap_query", h, C.byref(n), C.byref(nb), C.byref(rb))
        self.elem_num, self.nblocks, self.rbond_num = n.value, nb.value, rb.value

    def blocks(self):
        nb = self.nblocks
        q = (C.c_int * (3 * nb))()
        r, c, o = (C.c_int64 * nb)(), (C.c_int64 * nb)(), (C.c_int64 * nb)()
        call("tn_sectormap_blocks", self.h, q, r, c, o)
        return [((q[3 * i], q[3 * i + 1], q[3 * i + 2]), r[i], c[i], o[i]) for i in range(nb)]

    def __del__(self):
        try:
            capi.lib().tn_sectormap_destroy(self.h)
        except Exception:
            pass


def plan_check_permute(src: SectorMap, dst: SectorMap, rsp, src_host: np.ndarray) -> tuple[np.ndarray, int]:
    """Run the permute kernel's tile walk on the CPU (no GPU)."""
    s = np.ascontiguousarray(src_host, dtype=np.float64)
    d = np.full(dst.elem_num, np.nan)
    w = C.c_int64()
    call("tn_plan_check_permute", src.h, dst.h, int_array(rsp), s.ctypes.data, d.ctypes.data, C.byref(w))
    return d, w.value


def plan_check_views(src: SectorMap, dst: SectorMap, rsp, src_host: np.ndarray):
    """Build the permuted elements on the CPU through the operand views the
    FP64 GEMM would read instead of the permuted copy; None when the permute
    has no such views."""
    s = np.ascontiguousarray(src_host, dtype=np.float64)
    d = np.full(dst.elem_num, np.nan)
    ok = C.c_int()
    call("tn_plan_check_views", src.h, dst.h, int_array(rsp), s.ctypes.data, d.ctypes.data, C.byref(ok))
    return d if ok.value else None


def permute_device(src: SectorMap, dst: SectorMap, rsp, src_ptr: int, dst_ptr: int) -> None:
    call("tn_permute", None, src.h, dst.h, int_array(rsp), src_ptr, dst_ptr)


def permute_device_c128(src: SectorMap, dst: SectorMap, rsp, src_ptr: int, dst_ptr: int) -> None:
    """Complex (cflag) permute: elements are 16-byte (re, im) FP64 pairs."""
    call("tn_permute_c128", None, src.h, dst.h, int_array(rsp), src_ptr, dst_ptr)


def transpose_device_c128(src: SectorMap, dst: SectorMap, conj: bool, src_ptr: int, dst_ptr: int) -> None:
    """Complex transpose (conj=False) or cTranspose (conj=True) of every block;
    dst is the sector map of the bonds in transposed order."""
    call("tn_transpose_c128", None, src.h, dst.h, int(bool(conj)), src_ptr, dst_ptr)


def add_gate_c128(m: SectorMap, swaps, elem_ptr: int) -> None:
    """Complex addGate on a device buffer of 16-byte elements (in place)."""
    flat = [int(v) for p in swaps for v in p]
    call("tn_add_gate_c128", None, m.h, len(swaps), int_array(flat) if flat else None, elem_ptr)


def plan_check_permute_c128(src: SectorMap, dst: SectorMap, rsp, src_host: np.ndarray) -> tuple[np.ndarray, int]:
    """The complex permute's tile walk on the CPU (no GPU)."""
    s = np.ascontiguousarray(src_host, dtype=np.complex128)
    d = np.full(dst.elem_num, np.nan, dtype=np.complex128)
    w = C.c_int64()
    call("tn_plan_check_permute_c128", src.h, dst.h, int_array(rsp), s.ctypes.data, d.ctypes.data, C.byref(w))
    return d, w.value


def contract_sectors(mode, gemms, a_ptr: int, b_ptr: int, c_ptr: int) -> None:
    arr = (capi.SectorGemm * max(1, len(gemms)))(*[capi.SectorGemm(*g) for g in gemms])
    call("tn_contract_sectors", None, _mode(mode), len(gemms), arr, a_ptr, b_ptr, c_ptr)


def svd_sectors(sectors, a_ptr: int, u_ptr: int, s_ptr: int, vt_ptr: int, sweeps: bool = False):
    """Batched per-sector SVD; sectors are (M, N, a_off, u_off, s_off, vt_off)
    tuples, the pointers device addresses.  With sweeps=True returns the
    Jacobi sweep count of every sector (synchronous)."""
    n = len(sectors)
    arr = (capi.SvdSector * max(1, n))(*[capi.SvdSector(*t) for t in sectors])
    sw = (C.c_int * max(1, n))() if sweeps else None
    call("tn_svd_sectors", None, n, arr, a_ptr, u_ptr, s_ptr, vt_ptr, sw)
    return list(sw)[:n] if sweeps else None


def eigh_sectors(sectors, a_ptr: int, e_ptr: int, v_ptr: int, sweeps: bool = False):
    """Batched per-sector symmetric eigendecomposition (Block::eigh); sectors
    are (N, a_off, e_off, v_off) tuples, the pointers device addresses.
    Eigenvalues ascending, eigenvectors as rows.  With sweeps=True returns
    the Jacobi sweep count of every sector (synchronous)."""
    n = len(sectors)
    arr = (capi.EighSector * max(1, n))(*[capi.EighSector(*t) for t in sectors])
    sw = (C.c_int * max(1, n))() if sweeps else None
    call("tn_eigh_sectors", None, n, arr, a_ptr, e_ptr, v_ptr, sw)
    return list(sw)[:n] if sweeps else None


def svd_plan(M: int, N: int, max_cluster: int = 16) -> dict:
    P, b, L, sm = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
    call("tn_svd_plan", int(M), int(N), int(max_cluster), C.byref(P), C.byref(b), C.byref(L), C.byref(sm))
    return {"P": P.value, "b": b.value, "L": L.value, "smem": sm.value}


def truncate_sectors(s_off, counts, s_ptr: int, chi: int):
    """Global truncation of sorted per-sector singular values (device, in
    place); returns (kept per sector, norm)."""
    n = len(s_off)
    o = (C.c_int64 * max(1, n))(*s_off)
    k = (C.c_int64 * max(1, n))(*counts)
    kept = (C.c_int64 * max(1, n))()
    norm = C.c_double()
    call("tn_truncate_sectors", None, n, o, k, s_ptr, int(chi), kept, C.byref(norm))
    return list(kept)[:n], norm.value


def autotune(on: bool) -> int:
    """Switch the FP64 GEMM autotuner of the default context; returns the
    number of sector-size histograms tuned so far."""
    n = C.c_int64()
    call("tn_autotune", None, int(bool(on)), C.byref(n))
    return n.value


def sync() -> None:
    call("tn_ctx_sync", None)


def set_stream(stream_handle: int) -> None:
    call("tn_ctx_set_stream", None, C.c_void_p(stream_handle))


def prof_enable(on: bool) -> None:
    call("tn_prof_enable", None, int(bool(on)))


def prof_read() -> dict:
    cap = 64
    names = C.create_string_buffer(32 * cap)
    ms, by, fl = (C.c_double * cap)(), (C.c_double * cap)(), (C.c_double * cap)()
    la = (C.c_int64 * cap)()
    n = C.c_int()
    call("tn_prof_read", None, cap, names, ms, la, by, fl, C.byref(n))
    out = {}
    for i in range(n.value):
        nm = names.raw[32 * i : 32 * i + 32].split(b"\0")[0].decode()
        out[nm] = {"ms": ms[i], "launches": la[i], "bytes": by[i], "flops": fl[i]}
    return out


def launch_count() -> int:
    n = C.c_int64()
    call("tn_ctx_launch_count", None, C.byref(n))
    return n.value


class UniTensor:
    """Handle to a device-resident uni10::UniTensor."""

    def __init__(self, bonds=None, labels=None, elem=None, _h=None):
        if _h is not None:
            self.h = _h
        else:
            h = C.c_void_p()
            call("tn_tensor_create", None, *pack_bonds(bonds), C.byref(h))
            self.h = h
            if labels is not None:
                self.set_label(labels)
            if elem is not None:
                self.set_elem(elem)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                capi.lib().tn_tensor_destroy(self.h)
        except Exception:
            pass

    # -- elements
    def elem_num(self) -> int:
        n = C.c_int64()
        call("tn_tensor_device_elem", self.h, None, C.byref(n))
        return n.value

    def device_ptr(self) -> int:
        p = C.c_void_p()
        call("tn_tensor_device_elem", self.h, C.byref(p), None)
        return p.value or 0

    def set_elem(self, a) -> None:
        a = np.ascontiguousarray(a, dtype=np.float64)
        call("tn_tensor_set_elem", self.h, a.ctypes.data, a.size)

    def set_elem_host_ptr(self, ptr: int, n: int) -> None:
        call("tn_tensor_set_elem", self.h, ptr, n)

    def set_elem_host_ptr_async(self, ptr: int, n: int) -> None:
        """setElem from host memory without waiting: the buffer (pinned, for
        an overlapping copy) must stay unchanged until a synchronising call."""
        call("tn_tensor_set_elem_async", self.h, ptr, n)

    def get_elem(self) -> np.ndarray:
        out = np.empty(self.elem_num())
        call("tn_tensor_get_elem", self.h, out.ctypes.data, out.size)
        return out

    def get_elem_host_ptr(self, ptr: int, n: int) -> None:
        """getElem into caller-owned host memory (e.g. a pinned buffer) of n doubles."""
        call("tn_tensor_get_elem", self.h, ptr, n)

    def put_block(self, qnum, mat, diag: bool = False) -> None:
        """UniTensor::putBlock(qnum, Matrix): mat is a rows x cols array, or
        with diag=True the diagonal of a rows x cols matrix given as
        (rows, cols, values)."""
        q = int_array(list(qnum))
        if diag:
            rows, cols, vals = mat
            v = np.ascontiguousarray(vals, dtype=np.float64)
            call("tn_tensor_put_block", self.h, q, int(rows), int(cols), 1, v.ctypes.data, v.size)
        else:
            m = np.ascontiguousarray(mat, dtype=np.float64)
            call("tn_tensor_put_block", self.h, q, m.shape[0], m.shape[1], 0, m.ctypes.data, m.size)

    @staticmethod
    def load(path: str) -> "UniTensor":
        """UniTensor(fname): the reference's binary layout (current or older)."""
        h = C.c_void_p()
        call("tn_tensor_load", None, str(path).encode(), C.byref(h))
        return UniTensor(_h=h)

    def save(self, path: str) -> None:
        """UniTensor::save in the reference's binary layout."""
        call("tn_tensor_save", self.h, str(path).encode())

    def is_diagonal(self) -> bool:
        d = C.c_int()
        call("tn_tensor_is_diagonal", self.h, C.byref(d))
        return bool(d.value)

    # -- labels / bonds
    def set_label(self, labels) -> None:
        call("tn_tensor_set_label", self.h, len(labels), int_array(labels))

    def labels(self) -> list[int]:
        n = C.c_int()
        call("tn_tensor_get_labels", self.h, None, C.byref(n))
        buf = (C.c_int * max(1, n.value))()
        call("tn_tensor_get_labels", self.h, buf, C.byref(n))
        return list(buf[: n.value])

    def bonds(self):
        nb = C.c_int()
        cap = 4096
        bt, nq = (C.c_int * 64)(), (C.c_int * 64)()
        q, d = (C.c_int * (3 * cap))(), (C.c_int * cap)()
        call("tn_tensor_bonds", self.h, C.byref(nb), bt, nq, q, d, cap)
        out, r = [], 0
        for b in range(nb.value):
            runs = []
            for _ in range(nq[b]):
                runs.append((q[3 * r], q[3 * r + 1], q[3 * r + 2], d[r]))
                r += 1
            out.append((bt[b], runs))
        return out

    def sector_map(self) -> SectorMap:
        return SectorMap(self.bonds())

    # -- the path
    def permute(self, new_labels, in_bond_num: int) -> "UniTensor":
        call("tn_tensor_permute", self.h, len(new_labels), int_array(new_labels), in_bond_num)
        return self

    def add_gate(self, swaps) -> "UniTensor":
        """UniTensor::addGate: negate the sub-blocks whose swapped bond pairs
        carry an odd number of (odd, odd) fermionic parities (in place)."""
        flat = [int(v) for p in swaps for v in p]
        call("tn_tensor_add_gate", self.h, len(swaps), int_array(flat) if flat else None)
        return self

    def transpose(self) -> "UniTensor":
        call("tn_tensor_transpose", self.h)
        return self

    def combine_bond(self, labels) -> "UniTensor":
        call("tn_tensor_combine_bond", self.h, len(labels), int_array(labels))
        return self

    def copy(self) -> "UniTensor":
        h = C.c_void_p()
        call("tn_tensor_copy", self.h, C.byref(h))
        return UniTensor(_h=h)

    def scale(self, a: float) -> "UniTensor":
        call("tn_tensor_scale", self.h, C.c_double(a))
        return self

    def svd_truncate(self, chi: int):
        """Block SVDs truncated to the chi largest singular values over all
        blocks and normalised; returns (U, S, VT, norm) (the U(1) iTEBD update)."""
        u, sv, vt = C.c_void_p(), C.c_void_p(), C.c_void_p()
        norm = C.c_double()
        call("tn_tensor_svd_truncate", self.h, int(chi), C.byref(u), C.byref(sv), C.byref(vt), C.byref(norm))
        return UniTensor(_h=u), UniTensor(_h=sv), UniTensor(_h=vt), norm.value


def contract(a: UniTensor, b: UniTensor, fast: bool = False, mode="fp64") -> UniTensor:
    h = C.c_void_p()
    call("tn_contract", a.h, b.h, int(bool(fast)), _mode(mode), C.byref(h))
    return UniTensor(_h=h)


def contract_sectors_loop(mode, gemms, a_ptr: int, b_ptr: int, c_ptr: int) -> None:
    """The sector GEMMs one launch each (the reference's per-sector loop), in C++."""
    arr = (capi.SectorGemm * max(1, len(gemms)))(*[capi.SectorGemm(*g) for g in gemms])
    call("tn_contract_sectors_loop", None, _mode(mode), len(gemms), arr, a_ptr, b_ptr, c_ptr)


class Batch:
    """n independent contractions a[i] . b[i] with persistent operands and
    outputs: launch() is one grouped launch on a work list planned once;
    capture()/replay() run it as one CUDA graph."""

    def __init__(self, As, Bs):
        n = len(As)
        a = (C.c_void_p * max(1, n))(*[t.h.value for t in As])
        b = (C.c_void_p * max(1, n))(*[t.h.value for t in Bs])
        h = C.c_void_p()
        call("tn_batch_create", n, a, b, C.byref(h))
        self.h, self.n = h, n

    def __del__(self):
        try:
            capi.lib().tn_batch_destroy(self.h)
        except Exception:
            pass

    def put(self, i: int, a: "UniTensor", b: "UniTensor") -> None:
        call("tn_batch_put", self.h, int(i), a.h, b.h)

    def launch(self, mode="fp64") -> None:
        call("tn_batch_launch", self.h, _mode(mode))

    def capture(self, mode="fp64") -> None:
        call("tn_batch_capture", self.h, _mode(mode))

    def replay(self) -> None:
        call("tn_batch_replay", self.h)

    def output(self, i: int) -> "UniTensor":
        h = C.c_void_p()
        call("tn_batch_output", self.h, int(i), C.byref(h))
        return UniTensor(_h=h)

    def sectors(self):
        n = C.c_int()
        call("tn_batch_sectors", self.h, 0, None, C.byref(n))
        arr = (capi.SectorGemm * max(1, n.value))()
        call("tn_batch_sectors", self.h, n.value, arr, C.byref(n))
        return [(g.M, g.N, g.K, g.a_off, g.b_off, g.c_off) for g in arr[: n.value]]


def contract_batch(As, Bs, mode="fp64") -> list:
    n = len(As)
    a = (C.c_void_p * max(1, n))(*[t.h.value for t in As])
    b = (C.c_void_p * max(1, n))(*[t.h.value for t in Bs])
    out = (C.c_void_p * max(1, n))()
    call("tn_contract_batch", n, a, b, _mode(mode), out)
    return [UniTensor(_h=C.c_void_p(out[i])) for i in range(n)]


def otimes(a: UniTensor, b: UniTensor, mode="fp64") -> UniTensor:
    h = C.c_void_p()
    call("tn_otimes", a.h, b.h, _mode(mode), C.byref(h))
    return UniTensor(_h=h)


class Network:
    def __init__(self, text: str):
        h = C.c_void_p()
        call("tn_network_create", None, text.encode(), C.byref(h))
        self.h = h

    def __del__(self):
        try:
            capi.lib().tn_network_destroy(self.h)
        except Exception:
            pass

    def put_tensor(self, name: str, t: UniTensor) -> None:
        call("tn_network_put_tensor", self.h, name.encode(), t.h)

    def launch(self, mode="fp64") -> UniTensor:
        h = C.c_void_p()
        call("tn_network_launch", self.h, _mode(mode), C.byref(h))
        return UniTensor(_h=h)

    def capture(self, mode="fp64") -> None:
        call("tn_network_capture", self.h, _mode(mode))

    def replay(self) -> None:
        call("tn_network_replay", self.h)

    def bind_host_input(self, name: str, ptr: int, n: int) -> None:
        """Pinned host buffer copied into tensor `name` at the start of every
        replay of the next captured graph."""
        call("tn_network_bind_host_input", self.h, name.encode(), ptr, n)

    def bind_host_output(self, ptr: int, n: int) -> None:
        """Pinned host buffer the result is copied into at the end of every
        replay of the next captured graph (0 unbinds)."""
        call("tn_network_bind_host_output", self.h, ptr, n)

    def output(self) -> UniTensor:
        h = C.c_void_p()
        call("tn_network_output", self.h, C.byref(h))
        return UniTensor(_h=h)

    def tree(self) -> str:
        buf = C.create_string_buffer(4096)
        call("tn_network_tree", self.h, buf, 4096)
        return buf.value.decode()
