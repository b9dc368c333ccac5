"""Continuous-batching server: every result is the same alone and in the mix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

fl = pytest.importorskip("fluidlets_gb300")
from fluidlets_gb300.geometry import biflagellate_shape, fibonacci_sphere, mean_nn_spacing  # noqa: E402
from fluidlets_gb300.serve import ResistanceRequest, SolveServer, SwimmerRequest, bucket_of  # noqa: E402


def requests(seed=0, n=10):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        N = int(rng.integers(150, 1400))
        pts = fibonacci_sphere(N) * np.array([rng.uniform(1, 3), 1, 1])
        wall = k % 2 == 1
        if wall:
            pts = pts + [0, 0, -pts[:, 2].min() + rng.uniform(0.1, 1.0)]
        eps = rng.uniform(0.2, 0.4) * mean_nn_spacing(pts)
        U = np.tile(rng.normal(size=3), (N, 1)) if k % 3 else np.cross(rng.normal(size=3), pts)
        out.append(ResistanceRequest(fl.WallStokeslet3D() if wall else fl.Stokeslet3D(), pts, U, eps))
    for t in (0.1, 0.6):
        B = np.linalg.qr(rng.normal(size=(3, 3)))[0]
        B *= np.sign(np.linalg.det(B))
        out.append(SwimmerRequest(biflagellate_shape(t), np.array([0.1, 0.2, 0.3]), B, 0.02))
    return out


def alone(r):
    if isinstance(r, ResistanceRequest):
        F, info = fl.resistance(r.kernel, r.points, r.velocities, r.eps, method="lu")
        return F
    return fl.swimming_problem(r.shape, r.x0, r.B, r.eps)


def check(r, res, ref):
    if isinstance(r, ResistanceRequest):
        assert res.residual < 1e-10, res.residual
        assert np.linalg.norm(res.value - ref) / np.linalg.norm(ref) < 1e-9
        assert res.bucket == bucket_of(len(r.points))
    else:
        st = res.value
        for a, b in ((st.U, ref.U), (st.Omega, ref.Omega), (st.forces, ref.forces)):
            assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-9


@pytest.mark.parametrize("graphs", [True, False])
def test_results_alone_and_in_the_mix(graphs):
    reqs = requests(1)
    refs = [alone(r) for r in reqs]
    with SolveServer(slots=4, graphs=graphs) as srv:
        futs = [srv.submit(r) for r in reqs]  # all at once: they overlap on the device
        res = [f.result(timeout=180) for f in futs]
        # resubmit in reverse order while others are still queued: still the same results
        futs2 = [srv.submit(r) for r in reversed(reqs)]
        res2 = [f.result(timeout=180) for f in futs2][::-1]
        stats = dict(srv.stats)
    if graphs:
        assert stats["capture_errors"] == [] and stats["graph_replays"] > 0, stats
    else:
        assert stats["graph_replays"] == 0
    for r, x, x2, ref in zip(reqs, res, res2, refs):
        check(r, x, ref)
        check(r, x2, ref)
    assert len({x.slot for x in res}) > 1  # work was spread over several slots


def test_small_budget_still_serves_everything():
    reqs = requests(2, n=6)
    refs = [alone(r) for r in reqs]
    with SolveServer(slots=3, hbm_budget_gb=0.3) as srv:
        res = [f.result(timeout=180) for f in [srv.submit(r) for r in reqs]]
    for r, x, ref in zip(reqs, res, refs):
        check(r, x, ref)


def test_batched_groups_match_alone():
    """Requests of one bucket (640 points) submitted together are factored in groups of up to
    four, one replay of the batched graph per group; each result equals the request solved
    alone, and the wall requests (another plan key) never share a group with the free ones."""
    rng = np.random.default_rng(7)
    reqs = []
    for k in range(10):
        N = int(rng.integers(520, 641))
        pts = fibonacci_sphere(N) * np.array([rng.uniform(1, 2), 1, 1])
        wall = k % 3 == 2
        if wall:
            pts = pts + [0, 0, -pts[:, 2].min() + rng.uniform(0.1, 1.0)]
        eps = rng.uniform(0.2, 0.4) * mean_nn_spacing(pts)
        U = np.tile(rng.normal(size=3), (N, 1))
        reqs.append(ResistanceRequest(fl.WallStokeslet3D() if wall else fl.Stokeslet3D(), pts, U, eps))
    refs = [alone(r) for r in reqs]
    with SolveServer(slots=2, lu="tf32", batch=4) as srv:
        res = [f.result(timeout=180) for f in [srv.submit(r) for r in reqs]]
        stats = dict(srv.stats)
    assert stats["capture_errors"] == [], stats
    assert max(stats["groups"]) > 1, stats
    for r, x, ref in zip(reqs, res, refs):
        check(r, x, ref)
        assert x.bucket == 640
    assert any(x.batch > 1 for x in res)
