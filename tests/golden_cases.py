"""Shared loaders for the reference's known-answer cases (tests/golden)."""
import json
import os

import numpy as np

from oracle import pyoracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases():
    with open(os.path.join(GOLDEN, "reference_cases.json")) as f:
        return json.load(f)["cases"]


def case_ids():
    return ["%s@%s" % (c["name"], c["source"].split(":")[-1]) for c in cases()]


def triplets_for(case):
    """Triplet input of a case as (nor, noc, rows, cols, vals) via the oracle's
    loaders (Matrix/Triplet.hpp), or None for a Poisson case."""
    inp = case["input"]
    if inp["kind"] == "mm":
        return O.load_mm(os.path.join(GOLDEN, "matrices", inp["file"]), inp["has_data"], inp["symmetric"])
    if inp["kind"] == "bin":
        return O.load_bin(os.path.join(GOLDEN, "matrices", inp["file"]), inp["size"], inp["symmetric"])
    return None


def boost_close(a, b, tol):
    """Boost.Test floating-point `==` under tolerance(tol): strong relative
    closeness |a-b| <= tol*|a| and |a-b| <= tol*|b| (exact equality passes)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b)
    return (a == b) | ((d <= tol * np.abs(a)) & (d <= tol * np.abs(b)))


def ref_outputs():
    return np.load(os.path.join(GOLDEN, "ref_outputs.npz"))
