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


def stats_cases():
    """Square matrices for the calc_stats figures (Util_Scripts/calc_stats.cpp),
    built deterministically from the oracle's generators and the reference's
    input fixtures: list of (name, nor, rows, cols, vals)."""
    out = []
    for m, n in [(3, 3), (64, 48), (100, 100), (129, 1), (256, 256)]:
        r, c, v = O.triplet_poisson(m, n)
        out.append(("poisson_%dx%d" % (m, n), m * n, r, c, v))
    seen = set()
    for case in cases():
        inp = case["input"]
        if inp["kind"] == "poisson" or inp.get("file") in seen:
            continue
        seen.add(inp.get("file"))
        nor, noc, r, c, v = triplets_for(case)
        if nor == noc:
            out.append((inp["file"].replace(".", "_"), nor, r, c, v))
    for n, seed, kind in [(5000, 3, 0), (20000, 4, 1)]:
        A = O.random_crs(n, seed, kind=kind, mean=12.0, max_len=3000, band_half=256)
        rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(A.row_start))
        out.append(("random_%d_%d" % (n, seed), n, rows, A.col_ind, A.data))
    # an unbalanced block row: 4096 x 4096 (512-wide blocks), rows 0..511 get
    # 40 extra columns each on top of the Poisson stencil
    r, c, v = O.triplet_poisson(64, 64)
    er = np.repeat(np.arange(512, dtype=np.int32), 40)
    ec = ((np.arange(er.size, dtype=np.int64) * 97 + 1000) % 4096).astype(np.int32)
    out.append(("heavy_block_row", 4096, np.concatenate([r, er]), np.concatenate([c, ec]),
                np.concatenate([v, np.ones(er.size)])))
    return out


def ref_stats():
    with open(os.path.join(GOLDEN, "ref_stats.json")) as f:
        return json.load(f)["cases"]
