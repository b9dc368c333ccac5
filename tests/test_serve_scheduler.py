"""Scheduling of the solve server, on the host only (device work replaced by fakes):
admission by the HBM budget, eviction of idle plans, bucket affinity, grouping of same-key
requests for the batched graphs, no deadlock."""
import threading
import time

import numpy as np
import pytest

import fluidlets_gb300 as fl
from fluidlets_gb300.serve import ResistanceRequest, Result, SolveServer, SwimmerRequest, bucket_of, plan_bytes


class _Plan:
    def __init__(self, nbp, kind):
        self.nbp, self.kind = nbp, kind


class FakeServer(SolveServer):
    def __init__(self, *a, **k):
        self.peak = 0
        self.switches = 0
        self.concurrent = 0
        self.max_concurrent = 0
        self._lock2 = threading.Lock()
        super().__init__(*a, **k)

    def _device(self):
        return 0

    def _make_stream(self):
        return None

    def _run_group(self, slot, stream, reqs, b, plan, cap=1):
        with self._lock2:
            self.concurrent += 1
            self.max_concurrent = max(self.max_concurrent, self.concurrent)
        with self._cv:
            self.peak = max(self.peak, self._used)
            if plan is None:
                plan = _Plan(b, 0)
                plan.cap = cap
                if isinstance(reqs[0], ResistanceRequest):
                    self.switches += 1
        assert len(reqs) <= plan.cap
        time.sleep(0.001)
        with self._lock2:
            self.concurrent -= 1
        return [Result(None, 0.0, 0, 0, 0, slot, b) for _ in reqs], plan


def mix(n, seed, sizes=(200, 700, 1500, 3000)):
    rng = np.random.default_rng(seed)
    out = []
    shape = fl.SwimmerShape(np.zeros((50, 3)), np.zeros((50, 3)), np.zeros((200, 3)))
    for _ in range(n):
        if rng.random() < 0.25:
            out.append(SwimmerRequest(shape, np.zeros(3), np.eye(3), 0.1))
        else:
            N = int(rng.choice(sizes))
            out.append(ResistanceRequest(fl.Stokeslet3D(), np.zeros((N, 3)), np.zeros((N, 3)), 0.1))
    return out


@pytest.mark.parametrize("budget_gb", [0.05, 0.3, 1.0, 150.0])
def test_everything_completes_within_the_budget(budget_gb):
    reqs = mix(200, 1)
    with FakeServer(slots=4, hbm_budget_gb=budget_gb) as srv:
        futs = [srv.submit(r) for r in reqs]
        res = [f.result(timeout=60) for f in futs]
        peak, used = srv.peak, srv._used
    assert len(res) == len(reqs)
    largest = max(plan_bytes(bucket_of(len(r.points))) for r in reqs if isinstance(r, ResistanceRequest))
    # over budget only while a single request larger than the budget runs alone
    assert peak <= max(budget_gb * 2**30, largest + 16 * 156**2 + (64 << 20))
    assert used >= 0


def test_tight_budget_serializes_and_large_budget_overlaps():
    reqs = mix(120, 2)
    with FakeServer(slots=4, hbm_budget_gb=0.05) as srv:
        [f.result(timeout=60) for f in [srv.submit(r) for r in reqs]]
        tight = srv.max_concurrent
    with FakeServer(slots=4, hbm_budget_gb=150.0) as srv:
        [f.result(timeout=60) for f in [srv.submit(r) for r in reqs]]
        wide = srv.max_concurrent
    assert tight <= 2 and wide >= 3


def test_plan_pool_limits_replanning():
    reqs = mix(300, 3, sizes=(500, 2500))  # two buckets
    with FakeServer(slots=4, hbm_budget_gb=150.0, lookahead=16) as srv:
        [f.result(timeout=60) for f in [srv.submit(r) for r in reqs]]
        switches = srv.switches
    n_res = sum(isinstance(r, ResistanceRequest) for r in reqs)
    assert switches <= 2 * 4 + 2  # at most one plan per bucket and slot, not one per request
    assert n_res > 100


class _Stream:
    def synchronize(self):
        pass


def test_autotuner_keeps_the_fastest_candidate_that_converges(monkeypatch):
    """The per-bucket autotuner times every precision x tile-width candidate on one plan and
    keeps the fastest whose residual meets rtol; with none converging it falls back to TF32."""
    import fluidlets_gb300.serve as sv

    cost = {"tf32": 0.012, "tf32:128": 0.018, "tf32:256": 0.009, "bf16": 0.006, "bf16:128": 0.003,
            "bf16:256": 0.015, "fp32": 0.020}
    resid = dict.fromkeys(cost, 1e-12)
    resid["bf16:128"] = 1e-6  # fastest, but does not converge
    tried = []

    class Plan:
        def __init__(self, kernel, nbp, mu, lu, stream, **kw):
            self.lu = lu

        def set_lu(self, lu):
            self.lu = lu
            tried.append(lu)

        def factor(self, X, e):
            time.sleep(cost[self.lu])

        def solve(self, U, rtol):
            return None, 4, 2, resid[self.lu]

    monkeypatch.setattr(sv, "BucketPlan", Plan)
    assert set(cost) == set(sv.TUNE_CANDIDATES)
    req = ResistanceRequest(fl.Stokeslet3D(), np.zeros((300, 3)), np.zeros((300, 3)), 0.1)
    with FakeServer(slots=1) as srv:
        assert srv._autotune(req, 384, _Stream(), None, None, None) == "bf16"
        assert srv.stats["tuned"] == {"0:384": "bf16"}
        assert sorted(tried) == sorted(sv.TUNE_CANDIDATES)
        for k in resid:
            resid[k] = 1e-3
        assert srv._autotune(req, 512, _Stream(), None, None, None) == "tf32"


class GroupServer(FakeServer):
    """Records the groups the scheduler forms (device work replaced by a short sleep)."""

    def __init__(self, *a, **k):
        self.groups = []
        super().__init__(*a, **k)

    def _run_group(self, slot, stream, reqs, b, plan, cap=1):
        with self._cv:
            self.groups.append([(self._group_key(r, b), b) for r in reqs])
            if plan is None:
                plan = _Plan(b, 0)
                plan.cap = cap
        assert len(reqs) <= plan.cap
        time.sleep(0.002)
        return [Result(None, 0.0, 0, 0, 0, slot, b) for _ in reqs], plan


def test_same_key_requests_are_grouped_up_to_the_batch():
    """Requests submitted together are grouped by plan key (kernel, bucket, mu, LU mode, one
    blob width), at most `batch` per group, only for buckets up to `batch_points`; every
    request completes once, with its group size in the result."""
    reqs = mix(160, 4, sizes=(300, 700, 3000))  # buckets 384, 768 and 3072 points
    with GroupServer(slots=2, lu="tf32", batch=4, batch_points=2304) as srv:
        futs = [srv.submit(r) for r in reqs]
        res = [f.result(timeout=60) for f in futs]
        groups, stats = srv.groups, dict(srv.stats)
    assert len(res) == len(reqs)
    sizes = [len(g) for g in groups]
    assert sum(sizes) == len(reqs) and max(sizes) == 4
    for g in groups:
        assert len({k for k, _ in g}) == 1  # one plan key per group
        if g[0][0][0] != "swim" and g[0][1] > 2304:  # large buckets run alone
            assert len(g) == 1
    # swimmers of one shape size are grouped too
    assert max(len(g) for g in groups if g[0][0][0] == "swim") > 1
    assert sum(stats["groups"].get(k, 0) * k for k in stats["groups"]) == len(reqs)
    assert {r.batch for r in res} >= {1, 4}


def test_untuned_and_fp32_buckets_are_not_grouped():
    reqs = [r for r in mix(80, 5, sizes=(300,)) if isinstance(r, ResistanceRequest)]
    for lu in ("auto", "fp32"):
        with GroupServer(slots=2, lu=lu, batch=4) as srv:
            [f.result(timeout=60) for f in [srv.submit(r) for r in reqs]]
            assert max(len(g) for g in srv.groups) == 1, lu


def test_group_capacity_shrinks_to_the_budget():
    """A new plan holds up to `batch` systems, as many as the budget has room for: under a
    budget of two and a half swimmer systems the groups hold at most two."""
    shape = fl.SwimmerShape(np.zeros((50, 3)), np.zeros((50, 3)), np.zeros((200, 3)))
    reqs = [SwimmerRequest(shape, np.zeros(3), np.eye(3), 0.1) for _ in range(40)]
    one = SolveServer._need(reqs[0], 0)
    with GroupServer(slots=1, batch=4, hbm_budget_gb=2.5 * one / 2**30) as srv:
        [f.result(timeout=60) for f in [srv.submit(r) for r in reqs]]
        assert 1 < max(len(g) for g in srv.groups) <= 2


def test_batch_size_is_checked():
    for bad in (0, 65):
        with pytest.raises(ValueError):
            FakeServer(slots=1, batch=bad)
