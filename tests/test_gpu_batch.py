"""Independent meshes solved at once (femgpu_solve_batch), needs a GB300.

The meshes are cubes of uneven sizes, each with its own log-normal coefficient, as in the
batched multi-mesh workload; every batch result must equal the same handle's own
setup + solve bit for bit (the same kernels on its own stream)."""
import numpy as np
import pytest

import femgpu
from femgpu import meshes

pytestmark = pytest.mark.gpu


def problem(n, seed, **opts):
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(n, sigma=1.0, kappa_seed=seed, f_seed=1000 + seed)
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=300, flexibleCG=1, seed=1, **opts)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    b = np.where(mask.astype(bool), 0.0, s.load_vector(f))
    return s, b


@pytest.mark.parametrize("threads", [0, 1, 3])
def test_batch_matches_single_solves(threads):
    sizes = np.random.default_rng(7).integers(3, 11, size=6)
    probs = [problem(int(n), 8 + i) for i, n in enumerate(sizes)]
    xs, stats, status = femgpu.solve_batch([p[0] for p in probs], [p[1] for p in probs], threads=threads)
    assert status == 0
    for (s, b), x, st in zip(probs, xs, stats):
        assert st["relres"] <= 1e-8 and st["iterations"] > 0
        s.setup()
        x1, st1 = s.solve(b)
        assert np.array_equal(x, x1)
        assert st1["iterations"] == st["iterations"]


def test_batch_rejects_repeated_handles():
    s, b = problem(3, 8)
    xs, stats, status = femgpu.solve_batch([s, s], [b, b], check=False)
    assert status == 1  # FEMGPU_ERR_INVALID, before any work


def test_batch_attempts_every_problem():
    good, b = problem(4, 9)
    empty = femgpu.Solver(solverType=1)  # no operator
    xs, stats, status = femgpu.solve_batch([empty, good], [np.ones(8), b], x0s=[np.zeros(8), np.zeros(good.n)],
                                           check=False)
    assert status != 0
    assert stats[1]["relres"] <= 1e-8  # the later problem was still solved
    good.setup()
    x1, _ = good.solve(b)
    assert np.array_equal(xs[1], x1)


def test_batch_rejects_handles_on_one_stream():
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    p1 = problem(3, 8, stream=stream.cuda_stream)
    p2 = problem(4, 9, stream=stream.cuda_stream)
    xs, stats, status = femgpu.solve_batch([p1[0], p2[0]], [p1[1], p2[1]], check=False)
    assert status == 1  # FEMGPU_ERR_INVALID: their PCG captures would share the stream


def test_batch_graph_is_kept_and_recaptured():
    # second call: the kept graph (same handles, same hierarchies); third: new hierarchies
    # (setup again) recaptured into the same graph; a zero right-hand side skips its loop
    sizes = np.random.default_rng(3).integers(3, 9, size=5)
    probs = [problem(int(n), 20 + i) for i, n in enumerate(sizes)]
    solvers, bs = [p[0] for p in probs], [p[1] for p in probs]
    bs[2] = np.zeros_like(bs[2])
    first, _, status = femgpu.solve_batch(solvers, bs)
    assert status == 0
    for setup in (False, True):
        xs, stats, status = femgpu.solve_batch(solvers, bs, setup=setup)
        assert status == 0
        for x, x0 in zip(xs, first):
            assert np.array_equal(x, x0)
    assert stats[2]["iterations"] == 0 and not xs[2].any()
    for s, b, x in zip(solvers, bs, xs):
        x1, st1 = s.solve(b)
        assert np.array_equal(x, x1)


def test_batch_host_threads_match_the_graph(monkeypatch):
    sizes = np.random.default_rng(4).integers(3, 9, size=4)
    probs = [problem(int(n), 30 + i) for i, n in enumerate(sizes)]
    solvers, bs = [p[0] for p in probs], [p[1] for p in probs]
    xg, sg, _ = femgpu.solve_batch(solvers, bs)
    monkeypatch.setenv("FEMGPU_HOST_LOOP", "1")
    xt, st, _ = femgpu.solve_batch(solvers, bs)
    for a, b_, u, v in zip(xg, xt, sg, st):
        assert np.array_equal(a, b_) and u["iterations"] == v["iterations"]
