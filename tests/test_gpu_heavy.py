"""Rows the column-range planner cannot split (upper-bound mode) and the same
rows in the exact layout: a column that collects more products than one piece
holds, and a row of more pieces than the planner keeps.  Both take the
global-slab sort and must still equal the serial reference product bit for bit
(spgemm_common.cpp:131-178)."""
from __future__ import annotations

import numpy as np
import pytest

import spgemm_gb300 as sg
from helpers import csr_bits_equal, explain_diff

pytestmark = pytest.mark.gpu


def hot_column_case(seed: int = 1):
    """One output row whose column 5 collects 20,000 products (one bucket above
    the piece size), the rest spread; plus ordinary rows."""
    rng = np.random.default_rng(seed)
    nb = 20000
    lens = rng.integers(1, 4, size=nb)
    b_rows = []
    for i in range(nb):
        cols = [5] + list(rng.integers(0, 3000, size=int(lens[i])))
        b_rows.append(cols)
    rp = np.zeros(nb + 1, dtype=np.int64)
    rp[1:] = np.cumsum([len(c) for c in b_rows])
    b = sg.Csr(nb, 3000, rp, np.concatenate(b_rows).astype(np.int32),
               rng.integers(-4, 5, size=int(rp[-1])).astype(np.float64) * 0.25)
    a_rows = [np.arange(nb), rng.integers(0, nb, size=50), rng.integers(0, nb, size=7)]
    arp = np.zeros(4, dtype=np.int64)
    arp[1:] = np.cumsum([len(r) for r in a_rows])
    a = sg.Csr(3, nb, arp, np.concatenate(a_rows).astype(np.int32), rng.uniform(-1, 1, size=int(arp[-1])))
    return a, b


def many_pieces_case(seed: int = 2):
    """One output row of 4.5 M products spread over 2^20 columns: more than the
    planner's 256 pieces."""
    rng = np.random.default_rng(seed)
    b = sg.synth_uniform(4500, 1 << 20, 1000, seed=seed)
    a = sg.Csr.from_arrays(2, 4500, [0, 4500, 4510], np.concatenate([rng.permutation(4500),
                                                                    rng.integers(0, 4500, size=10)]),
                           rng.uniform(-1, 1, size=4510))
    return a, b


@pytest.mark.parametrize("mode", ["upper_bound", "exact"])
@pytest.mark.parametrize("case", ["hot_column", "many_pieces"])
def test_unsplittable_rows(port, mode, case):
    a, b = hot_column_case() if case == "hot_column" else many_pieces_case()
    want = port.serial_spgemm(a, b)
    with sg.Engine(0, mode=mode) as eng:
        got = eng.multiply(a, b)
        t = eng.last_timings()
    assert t["bin_rows"]["heavy"] >= 1
    assert csr_bits_equal(got, want), explain_diff(got, want)
