"""GPU tests of the bin autotuner (spg_tune): every alternative team shape
gives the same bits as the default ones (the serial reference product,
spgemm_common.cpp:131-178), and tuning only changes speed."""
from __future__ import annotations

import pytest

from helpers import csr_bits_equal, explain_diff, row_sizes_for_bins
from spgemm_gb300 import SpgError, synth_powerlaw, synth_uniform

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["bins", "powerlaw", "uniform"])
def test_alternative_shapes_are_bit_identical(engine, case):
    if case == "bins":
        a, b = row_sizes_for_bins(5)
    elif case == "powerlaw":
        a = synth_powerlaw(30000, 24.0, 1.2, 5000, 512, 0.7, seed=2)
        b = a
    else:
        a, b = synth_uniform(20000, 20000, 8, 48, seed=3), synth_uniform(20000, 20000, 8, 48, seed=4)
    engine.bin_variants = [0] * 20
    want = engine.multiply(a, b)
    engine.bin_variants = [1] * 20
    try:
        got = engine.multiply(a, b)
    finally:
        engine.bin_variants = [0] * 20
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_tune_keeps_results(engine, port):
    a = synth_powerlaw(20000, 24.0, 1.2, 3000, 256, 0.7, seed=7)
    before = engine.multiply(a, a)
    rep = engine.tune(a, a, reps=2)
    try:
        assert set(rep["variants"]) <= {0, 1}
        assert engine.bin_variants == rep["variants"]
        assert rep["products"] == engine.scalar_multiplication_count(a, a)
        for name, v in rep["bins"].items():
            assert v["ms_default"] > 0 and v["ms_alt"] > 0
            # a kept alternative was a candidate: at least 3% faster with the bins one after the other
            assert not v["variant"] or v["ms_alt"] < 0.97 * v["ms_default"], (name, v)
        after = engine.multiply(a, a)
        assert csr_bits_equal(after, before), explain_diff(after, before)
    finally:
        engine.bin_variants = [0] * 20


def test_tune_on_one_stream_keeps_results():
    # bins on one stream: the candidates are kept without the confirmation pass
    from spgemm_gb300 import Engine
    a = synth_powerlaw(20000, 24.0, 1.2, 3000, 256, 0.7, seed=8)
    with Engine(0, bin_streams=1) as eng:
        before = eng.multiply(a, a)
        rep = eng.tune(a, a, reps=1)
        assert eng.bin_variants == rep["variants"]
        for name, v in rep["bins"].items():
            assert not v["variant"] or v["ms_alt"] < 0.97 * v["ms_default"], (name, v)
        after = eng.multiply(a, a)
        assert csr_bits_equal(after, before), explain_diff(after, before)


def test_set_bin_variants_rejects_bad_values(engine):
    with pytest.raises(SpgError):
        engine.bin_variants = [2] + [0] * 19
    assert engine.bin_variants == [0] * 20
