"""The package's host Triplet loaders (numpy restatements of
Matrix/Triplet.hpp:75-154 loadFromMM, :164-216 loadFromBin, :226-278
generatePoisson) give the same triplets, in the same order, as the oracle's
C loaders on every matrix file of the reference's known-answer cases."""
import os

import numpy as np
import pytest

from golden_cases import GOLDEN, cases
from oracle import pyoracle as O
from thesis_spmv_gb300.matrix import Triplet


def _file_cases():
    seen, out = set(), []
    for c in cases():
        inp = c["input"]
        if inp["kind"] in ("mm", "bin"):
            key = tuple(sorted(inp.items()))
            if key not in seen:
                seen.add(key)
                out.append(inp)
    return out


@pytest.mark.parametrize("inp", _file_cases(), ids=lambda i: "%s-%s" % (i["kind"], i["file"]))
def test_file_loader_matches_oracle(inp):
    path = os.path.join(GOLDEN, "matrices", inp["file"])
    if inp["kind"] == "mm":
        nor, noc, r, c, v = O.load_mm(path, inp["has_data"], inp["symmetric"])
        t = Triplet().loadFromMM(path, inp["has_data"], inp["symmetric"])
    else:
        nor, noc, r, c, v = O.load_bin(path, inp["size"], inp["symmetric"])
        t = Triplet().loadFromBin(path, inp["size"], inp["symmetric"])
    assert (t.row_size, t.col_size, t.nnz) == (nor, noc, r.size)
    assert np.array_equal(t.row_coord, r)
    assert np.array_equal(t.col_coord, c)
    assert np.array_equal(t.data, v)


@pytest.mark.parametrize("m,n", [(1, 1), (1, 7), (7, 1), (5, 3), (16, 16), (33, 9)])
def test_generate_poisson_matches_oracle(m, n):
    r, c, v = O.triplet_poisson(m, n)
    t = Triplet().generatePoisson(m, n)
    assert t.row_size == t.col_size == m * n
    assert np.array_equal(t.row_coord, r)
    assert np.array_equal(t.col_coord, c)
    assert np.array_equal(t.data, v)
