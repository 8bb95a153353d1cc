"""GPU tests of the serving loop (spg_server_create / spg_submit / spg_poll).

A served result must be bit-identical to the same product run alone through
spg_multiply (and so to the serial reference product, spgemm_common.cpp:131-178),
whatever else shares its batch; admission, error isolation, cancellation and
concurrent submitters are exercised on mixes of uneven products.
"""
from __future__ import annotations

import threading

import numpy as np
import pytest

from helpers import csr_bits_equal, explain_diff, random_csr, row_sizes_for_bins
from spgemm_gb300 import Csr, Server, synth_powerlaw, synth_uniform

pytestmark = pytest.mark.gpu


def request_mix(seed: int, n: int = 14):
    """Uneven products: tiny random, every-bin rows, power-law and uniform blocks."""
    rng = np.random.default_rng(seed)
    pairs = []
    for i in range(n):
        kind = i % 4
        if kind == 0:
            m, k, c = (int(x) for x in rng.integers(1, 300, size=3))
            pairs.append((random_csr(m, k, rng.integers(0, 12, size=m), seed * 100 + i),
                          random_csr(k, c, rng.integers(0, 12, size=k), seed * 100 + i + 50)))
        elif kind == 1:
            pairs.append(row_sizes_for_bins(seed + i))
        elif kind == 2:
            a = synth_powerlaw(int(rng.integers(2000, 20000)), 24.0, 1.2, 2000, 256, 0.7, seed=seed + i)
            pairs.append((a, a))
        else:
            r = int(rng.integers(1000, 8000))
            pairs.append((synth_uniform(r, r, 4, 64, seed=seed + i), synth_uniform(r, r, 4, 64, seed=seed + i + 1)))
    return pairs


def serve_all(server, pairs, wait_ms=-1):
    tickets = [server.submit(a, b) for a, b in pairs]
    out = []
    for t in tickets:
        st, res, info = server.poll(t, wait_ms)
        out.append((st, res, info))
    return out


@pytest.mark.parametrize("lanes,max_batch", [(2, 4), (2, 256), (1, 1), (3, 2)])
def test_mix_equals_alone(engine, port, lanes, max_batch):
    pairs = request_mix(3)
    with Server(0, lanes=lanes, max_batch=max_batch, out="device") as srv:
        served = serve_all(srv, pairs)
        for (a, b), (st, res, info) in zip(pairs, served):
            assert st == "SPG_OK", info
            got = res.download()
            res.free()
            alone = engine.multiply(a, b)
            assert csr_bits_equal(got, alone), explain_diff(got, alone)
            assert info["latency_ms"] >= info["service_ms"] >= 0.0
            assert 1 <= info["batch_requests"] <= max_batch
    # the reference itself on the small ones
    for (a, b), (st, _, _) in list(zip(pairs, served))[:3]:
        want = port.serial_spgemm(a, b)
        assert csr_bits_equal(engine.multiply(a, b), want)


def test_device_operands_and_host_results(engine):
    pairs = request_mix(5, n=8)
    dev = [(a.to_device(), a.to_device() if b is a else b.to_device()) for a, b in pairs]
    with Server(0, lanes=2, max_batch=3, out="host") as srv:
        served = serve_all(srv, dev)
        for (a, b), (st, res, info) in zip(pairs, served):
            assert st == "SPG_OK", info
            got = res.download()
            res.free()
            assert csr_bits_equal(got, engine.multiply(a, b))
            assert info["products"] == engine.scalar_multiplication_count(a, b)


def test_budget_rejects_only_the_oversized_request(engine):
    small = random_csr(50, 40, 5, 1), random_csr(40, 30, 5, 2)
    big = synth_uniform(20000, 20000, 32, 32, seed=9)
    budget = 64 << 20  # 64 MiB: the big product needs ~36 B x 20.5M products
    with Server(0, lanes=2, max_batch=8, hbm_budget_bytes=budget) as srv:
        t_small = srv.submit(*small)
        t_big = srv.submit(big, big)
        t_small2 = srv.submit(*small)
        st, res, _ = srv.poll(t_small)
        assert st == "SPG_OK"
        res.free()
        st, res, info = srv.poll(t_big)
        assert st == "SPG_BUDGET_EXCEEDED" and res is None and "budget" in info["message"]
        st, res, _ = srv.poll(t_small2)
        assert st == "SPG_OK"
        assert csr_bits_equal(res.download(), engine.multiply(*small))
        res.free()


def test_bad_request_fails_alone(engine):
    good = [(random_csr(30, 20, 4, s), random_csr(20, 25, 4, s + 1)) for s in range(5)]
    bad_a = Csr.from_arrays(2, 3, [0, 1, 2], [0, 7], [1.0, 1.0])  # column 7 outside B's 3 rows
    bad_b = Csr.from_arrays(3, 2, [0, 1, 2, 3], [0, 1, 0], [1.0, 1.0, 1.0])
    mix = good[:2] + [(bad_a, bad_b)] + good[2:]
    with Server(0, lanes=1, max_batch=16) as srv:
        served = serve_all(srv, mix)
    names = [st for st, _, _ in served]
    assert names[2] in ("SPG_OUT_OF_RANGE_COLUMN", "SPG_INVALID_ARGUMENT")
    for i, (st, res, _) in enumerate(served):
        if i == 2:
            continue
        assert st == "SPG_OK"
        a, b = mix[i]
        assert csr_bits_equal(res.download(), engine.multiply(a, b))
        res.free()


def test_cancel_queued_requests():
    big = synth_uniform(40000, 40000, 32, 32, seed=4)
    small = random_csr(10, 10, 3, 1), random_csr(10, 10, 3, 2)
    with Server(0, lanes=1, max_batch=1) as srv:
        first = [srv.submit(big, big) for _ in range(3)]
        late = [srv.submit(*small) for _ in range(6)]
        cancelled = [srv.cancel(t) for t in late]
        assert all(c in ("SPG_OK", "SPG_NOT_READY") for c in cancelled)
        assert "SPG_OK" in cancelled  # the single lane is still busy with the big ones
        for t in first:
            st, res, _ = srv.poll(t)
            assert st == "SPG_OK"
            res.free()
        for t, c in zip(late, cancelled):
            st, res, _ = srv.poll(t)
            assert st == ("SPG_CANCELLED" if c == "SPG_OK" else "SPG_OK")
            if res is not None:
                res.free()
        assert srv.cancel(first[0]) == "SPG_INVALID_ARGUMENT"  # retired tickets are unknown


def test_poll_not_ready_then_ready(engine):
    big = synth_uniform(60000, 60000, 32, 32, seed=6)
    with Server(0, lanes=1, max_batch=1) as srv:
        t = srv.submit(big, big)
        st, res, _ = srv.poll(t, 0)
        assert st in ("SPG_NOT_READY", "SPG_OK")
        while st == "SPG_NOT_READY":
            assert res is None
            st, res, _ = srv.poll(t, 50)
        assert st == "SPG_OK" and res.nnz == engine.multiply(big, big).nnz
        res.free()


def test_concurrent_submitters(engine):
    pairs = request_mix(11, n=16)
    alone = [engine.multiply(a, b) for a, b in pairs]
    errors = []
    with Server(0, lanes=2, max_batch=5, out="host") as srv:
        def client(idx):
            try:
                for i in idx:
                    t = srv.submit(*pairs[i])
                    st, res, _ = srv.poll(t)
                    assert st == "SPG_OK"
                    got = res.download()
                    res.free()
                    assert csr_bits_equal(got, alone[i]), explain_diff(got, alone[i])
            except Exception as e:  # surfaced in the main thread
                errors.append(e)
        threads = [threading.Thread(target=client, args=(range(k, 16, 4),)) for k in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
    assert not errors, errors[0]
