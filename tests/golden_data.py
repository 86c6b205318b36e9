"""Loader for the golden fixtures generated by tests/golden/make_golden.py."""
import functools
import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@functools.lru_cache(maxsize=None)
def cases():
    with open(os.path.join(HERE, "cases.json")) as f:
        return {c["id"]: c for c in json.load(f)}


@functools.lru_cache(maxsize=None)
def arrays():
    with np.load(os.path.join(HERE, "arrays.npz")) as z:
        return {k: z[k] for k in z.files}


def arr(case_id, key):
    return arrays()[f"{case_id}/{key}"]


def bonds_of(meta):
    return [(t, [tuple(r) for r in runs]) for t, runs in meta["bonds"]]


@functools.lru_cache(maxsize=None)
def legacy():
    with np.load(os.path.join(HERE, "legacy.npz")) as z:
        d = {k: z[k] for k in z.files}
    d["_meta"] = json.loads(bytes(d["_meta"]).decode())
    return d
