"""Drive the compiled reference (oracle/_ref/ref_driver) from Python -- TEST ORACLE.

Used on the machine where the reference sources are present (oracle/_ref
is built from them by oracle/refbuild/Makefile) to pin the numpy
restatement and to write golden fixtures.  ``available()`` is False on
machines without the built reference; callers skip then.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

from . import uni10_io

HERE = os.path.dirname(os.path.abspath(__file__))
DRIVER = os.path.join(HERE, "_ref", "ref_driver")


def available() -> bool:
    return os.path.exists(DRIVER)


def bond_line(bond) -> str:
    btype, runs = bond
    parts = ["bond", "in" if btype == 1 else "out", str(len(runs))]
    for (u, p, f, d) in runs:
        parts += [str(u), str(p), str(f), str(d)]
    return " ".join(parts)


class RefSession:
    """Accumulates a ref_driver script; ``run()`` executes it and returns the
    saved tensors and timing lines."""

    def __init__(self):
        self.tmp = tempfile.TemporaryDirectory()
        self.lines: list[str] = []
        self.saves: dict[str, str] = {}
        self.files: dict[str, str] = {}

    def tensor(self, name: str, bonds, labels, elem) -> None:
        self.lines.append(f"tensor {name} {len(bonds)}")
        self.lines += [bond_line(b) for b in bonds]
        path = os.path.join(self.tmp.name, f"in_{name}.f64")
        np.ascontiguousarray(elem, dtype="<f8").tofile(path)
        self.lines.append(f"elems {name} {path} 0")
        self.lines.append("labels " + name + " " + " ".join(map(str, labels)))

    def cmd(self, line: str) -> None:
        self.lines.append(line)

    def network(self, out: str, net_text: str, puts: dict) -> None:
        path = os.path.join(self.tmp.name, f"net_{out}.net")
        with open(path, "w") as f:
            f.write(net_text)
        args = " ".join(f"{k} {v}" for k, v in puts.items())
        self.lines.append(f"network {out} {path} {args}")

    def save(self, name: str, key: str | None = None) -> None:
        path = os.path.join(self.tmp.name, f"out_{key or name}.bin")
        self.saves[key or name] = path
        self.lines.append(f"save {name} {path}")

    def svd(self, name: str, q, key: str) -> None:
        prefix = os.path.join(self.tmp.name, f"svd_{key}")
        self.files[key] = prefix
        self.lines.append(f"svd {name} {q[0]} {q[1]} {q[2]} {prefix}")

    def eigh(self, name: str, q, key: str) -> None:
        prefix = os.path.join(self.tmp.name, f"eigh_{key}")
        self.files[key] = prefix
        self.lines.append(f"eigh {name} {q[0]} {q[1]} {q[2]} {prefix}")

    def run(self, env=None) -> dict:
        script = os.path.join(self.tmp.name, "script.txt")
        with open(script, "w") as f:
            f.write("\n".join(self.lines) + "\n")
        e = dict(os.environ)
        if env:
            e.update(env)
        p = subprocess.run([DRIVER, script], capture_output=True, text=True, env=e)
        if p.returncode != 0:
            raise RuntimeError(f"ref_driver failed ({p.returncode}): {p.stderr[-2000:]}")
        out = {k: uni10_io.read_tensor(v) for k, v in self.saves.items()}
        for k, prefix in self.files.items():
            mats = []
            sufs = (".E", ".V") if os.path.exists(prefix + ".E") else (".U", ".S", ".VT")
            for suf in sufs:
                raw = np.fromfile(prefix + suf, dtype="<u8", count=2)
                m = np.fromfile(prefix + suf, dtype="<f8", offset=16)
                # a diagonal Matrix (the singular values) stores min(r, c) values
                mats.append(m if m.size != int(raw[0]) * int(raw[1]) else m.reshape(int(raw[0]), int(raw[1])))
            out[k] = mats
        out["_stdout"] = p.stdout
        return out
