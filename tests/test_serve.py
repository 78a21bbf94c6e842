"""Serving loop: requests answered by batched rounds get their own round's result;
admission by HBM budget; latency and throughput summary. CPU (emulation build)."""
import numpy as np
import pytest

from parafrost_gb300 import cnfgen, rounddump as rd
from parafrost_gb300.options import Options
from parafrost_gb300.serve import Server, estimate_footprint, poisson_load, summarize
from parafrost_gb300.sigma import Simplifier


def small_requests(n, seed=2):
    return [cnfgen.aig_unrolled(num_gates=60 + 7 * i, steps=2 + i % 4, seed=seed * 100 + i) for i in range(n)]


def own_round(lib, f, opts):
    s = Simplifier(opts, library=lib)
    s.awaken(*f)
    st = s.sigmify()
    out = rd.canonical_result(st.status, s.result() if st.status == 0 else None), st.phases_run
    s.close()
    return out


@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_serve_results(built, mode):
    opts = Options(all=1)
    reqs_f = small_requests(10)
    with Server(opts, mode=mode, library=built["emu"]) as srv:
        reqs = [srv.submit(f) for f in reqs_f]
        for r in reqs:
            assert r.wait(120)
    for f, r in zip(reqs_f, reqs):
        assert r.error is None
        want, ph = own_round(built["emu"], f, opts)
        assert rd.canonical_result(r.status, r.result) == want
        assert r.phases == ph
    if mode == "plain":
        assert all(b[0] >= 1 for b in srv.batches)


def test_serve_admission(built):
    reqs_f = small_requests(6, seed=3)
    need = [estimate_footprint(f[0], f[2].size - 1, f[1].size) for f in reqs_f]
    # room for about two requests per batch; a request above the budget is refused
    budget = max(need) * 2 + 1
    big = cnfgen.aig_unrolled(num_gates=400, steps=20, seed=9)
    assert estimate_footprint(big[0], big[2].size - 1, big[1].size) > budget
    srv = Server(Options(all=1), hbm_budget=budget, library=built["emu"], lanes=1)
    reqs = [srv.submit(f) for f in reqs_f]  # queued before the server starts: one admission pass
    refused = srv.submit(big)
    srv.start()
    for r in reqs:
        assert r.wait(120)
    srv.stop()
    assert refused.status == -2 and refused.error
    assert all(r.status in (0, 1) for r in reqs)
    assert all(b[2] <= budget for b in srv.batches)
    assert len(srv.batches) >= 2
    assert sum(b[0] for b in srv.batches) == len(reqs)
    assert srv.max_footprint > 0


def test_poisson_summary(built):
    pool = small_requests(4, seed=4)
    with Server(Options(all=1), library=built["emu"]) as srv:
        reqs = poisson_load(srv, pool, rate=400.0, num=16, seed=1)
    s = summarize(reqs, srv)
    assert s["served"] == 16 and s["failed"] == 0
    assert 0 < s["p50_ms"] <= s["p99_ms"]
    assert s["formulas_per_s"] > 0 and s["batches"] >= 1


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_serve_gpu(cuda_lib, mode):
    opts = Options(all=1)
    reqs_f = small_requests(12, seed=6) + [cnfgen.aig_unrolled(num_gates=5000, steps=6, seed=11)]
    with Server(opts, mode=mode, library=cuda_lib) as srv:
        reqs = poisson_load(srv, reqs_f, rate=2000.0, num=len(reqs_f), seed=2)
    for f, r in zip(reqs_f, reqs):
        assert r.error is None
        want, ph = own_round(cuda_lib, f, opts)
        assert rd.canonical_result(r.status, r.result) == want
        assert r.phases == ph


def test_serve_without_library_fails_requests():
    """A worker that cannot open its context answers every request with the error
    instead of leaving it waiting."""
    reqs_f = small_requests(3, seed=7)
    with Server(Options(all=1), library="/nonexistent/libsigma.so") as srv:
        reqs = [srv.submit(f) for f in reqs_f]
        for r in reqs:
            assert r.wait(30)
    assert all(r.status is not None and r.status < 0 and r.error for r in reqs)


def test_serve_lanes(built):
    """Small and large requests go to separate lanes; every result is still the
    request's own round."""
    opts = Options(all=1)
    small = small_requests(6, seed=8)
    large = [cnfgen.aig_unrolled(num_gates=300, steps=12, seed=12 + i) for i in range(2)]
    sizes = sorted(f[2].size - 1 for f in small + large)
    cut = (max(f[2].size - 1 for f in small) + min(f[2].size - 1 for f in large)) // 2
    assert max(f[2].size - 1 for f in small) < cut < min(f[2].size - 1 for f in large), sizes
    with Server(opts, library=built["emu"], small_clauses=cut) as srv:
        assert srv.lanes == 2 and srv.workers == 4
        assert {srv.lane_of(f) for f in small} == {0} and {srv.lane_of(f) for f in large} == {1}
        reqs = [srv.submit(f) for f in large + small]
        for r in reqs:
            assert r.wait(120)
    for f, r in zip(large + small, reqs):
        want, ph = own_round(built["emu"], f, opts)
        assert rd.canonical_result(r.status, r.result) == want
