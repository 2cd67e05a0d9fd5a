"""Serving: admission under the HBM budget (CPU), and on the GPU that every
request's result is the same alone and in the mix (bit for bit: the same
kernels on the same inputs), and agrees with the plain per-request path."""
import numpy as np
import pytest

from htr_gb300 import serve

from tests import util


def test_request_mix_is_seeded_and_poisson():
    a = serve.request_mix(400, rate=200.0, seed=3)
    b = serve.request_mix(400, rate=200.0, seed=3)
    assert [(r.kind, r.size, r.steps, r.arrival) for r in a] == [(r.kind, r.size, r.steps, r.arrival) for r in b]
    gaps = np.diff([0.0] + [r.arrival for r in a])
    assert 0.8 / 200 < gaps.mean() < 1.2 / 200
    assert {r.kind for r in a} == {"tube", "vortex", "box"}
    assert all(100 <= r.steps <= 2000 for r in a)


def test_admission_is_fifo_under_budget():
    reqs = [serve.Request(i, "box", 32, 0, 10, arrival=0.1 * i) for i in range(5)]
    size = lambda r: 10
    assert serve.admissible(reqs, now=0.25, used=0, budget=100, size=size) == 3
    assert serve.admissible(reqs, now=1.0, used=75, budget=100, size=size) == 2
    assert serve.admissible(reqs, now=1.0, used=95, budget=100, size=size) == 0
    big = [serve.Request(0, "box", 96, 0, 10, 0.0), serve.Request(1, "tube", 300, 0, 10, 0.0)]
    assert serve.admissible(big, now=1.0, used=0, budget=serve.estimate_bytes(big[0]) - 1) == 0


def test_round_selection_is_shortest_remaining_work_first():
    from types import SimpleNamespace as NS
    active = [NS(remaining=r, cells=c) for r, c in ((100, 1000), (5, 1000), (50, 10), (1, 5000), (5, 1000))]
    assert serve.round_selection(active, None) == active
    # least remaining work first: #2 (500), then #1, #3, #4 (5000 each, in
    # admission order), then #0
    assert serve.round_selection(active, 1) == [active[2]]
    assert serve.round_selection(active, 1010) == [active[1], active[2]]
    assert serve.round_selection(active, 2010) == [active[1], active[2], active[3]]
    assert serve.round_selection(active, 10 ** 9) == active


def test_estimate_covers_sizes():
    sizes = [serve.estimate_bytes(serve.Request(0, k, n, 0, 1, 0.0))
             for k, n in (("tube", 256), ("tube", 8192), ("vortex", 64), ("vortex", 512), ("box", 32), ("box", 96))]
    assert sizes[0] < sizes[1] and sizes[2] < sizes[3] and sizes[4] < sizes[5]
    assert sizes[5] < 2e9


def _small_mix():
    reqs = serve.request_mix(6, rate=2000.0, seed=11, steps=(2, 4), tube=(24, 40), vortex=(12, 16), box=(6, 8))
    kinds = [r.kind for r in reqs]
    assert len(set(kinds)) >= 2
    return reqs


@pytest.mark.gpu
def test_results_same_alone_and_in_mix():
    mix = _small_mix()
    server = serve.Server(streams=4)
    server.run(mix)
    for r in mix:
        alone = serve.Request(r.rid, r.kind, r.size, r.seed, r.steps, 0.0)
        serve.Server(streams=1).run([alone])
        assert np.array_equal(alone.result, r.result), (r.kind, r.size)


@pytest.mark.gpu
def test_server_matches_plain_path_and_budget():
    mix = _small_mix()
    budget = 2 * max(serve.estimate_bytes(r) for r in mix)
    server = serve.Server(streams=4, hbm_budget=budget)
    server.run(mix)
    assert server.peak <= budget and all(r.done is not None for r in mix)
    assert server.over_estimate <= 1.0
    plain = [serve.Request(r.rid, r.kind, r.size, r.seed, r.steps, r.arrival) for r in mix]
    serve.run_plain(plain)
    for a, b in zip(mix, plain):
        ratio, info = util.pointwise(a.result, b.result, "Conserved")
        assert ratio <= 1.0, (a.kind, a.size, info)
