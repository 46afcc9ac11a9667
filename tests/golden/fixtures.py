"""Loaders for the committed golden fixtures (see make_golden.py)."""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def modp_cases():
    """[(name, A uint64, p, R uint64, pivots)] from modp_cases.npz."""
    z = np.load(os.path.join(HERE, "modp_cases.npz"))
    out = []
    for name in z["__names__"]:
        name = str(name)
        out.append((name, z[f"{name}__A"], int(z[f"{name}__p"][0]), z[f"{name}__R"],
                    [int(x) for x in z[f"{name}__piv"]]))
    return out


def float_cases():
    z = np.load(os.path.join(HERE, "float_cases.npz"))
    return [(str(n), z[f"{n}__A"], z[f"{n}__R"]) for n in z["__names__"]]


def config1():
    with open(os.path.join(HERE, "config1.json")) as f:
        return json.load(f)


def known_result_4096():
    return np.load(os.path.join(HERE, "known_result_4096_4097_2to32m19.npy"))


def golden_4096_input():
    """The reference test's input: numpy legacy seed 0, uint32 residues mod
    2^31-19, 4097 x 4097 drawn, last row dropped (4096 x 4097)."""
    rs = np.random.RandomState(0)
    return rs.randint(2**31 - 19, size=(4097, 4097), dtype=np.uint32)[:-1, :], 2**31 - 19


def nullspace(size: str):
    z = np.load(os.path.join(HERE, f"nullspace_{size}_2147483647.npz"))
    return {k: z[k] for k in z.files}


class Field:
    """Minimal field descriptor for dict-form points (name, characteristic)."""

    def __init__(self, name, characteristic):
        self.name = name
        self.characteristic = characteristic

    def __contains__(self, x):
        return False


def loader_cases():
    with open(os.path.join(HERE, "loader_cases.json")) as f:
        meta = json.load(f)
    z = np.load(os.path.join(HERE, "loader_cases.npz"))
    cases = []
    for fm in meta["fields"]:
        k, p = fm["index"], fm["p"]
        pts = {"field": Field(fm["field"], p)}
        for key in meta["point_keys"]:
            arr = z[f"f{k}_pt_{key}"]
            pts[key] = np.array([int(v) for v in arr], dtype=object) if p > 0 else arr
        As = [z[f"f{k}_A{t}"] for t in range(fm["n_matrices"])]
        cases.append((fm["field"], p, pts, As))
    return meta["prefactors"], meta["ansatze"], cases
