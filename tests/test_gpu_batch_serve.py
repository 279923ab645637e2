"""Batched stepping, re-batching, the autotuner and the continuous-batching
server on the GPU.  A grid's result must not depend on what else shares its
batch: states are compared bitwise against the same grid advanced alone."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from torch_gb300 import autotune  # noqa: E402
from torch_gb300.batch import Batch, Grid  # noqa: E402
from torch_gb300.serve import Server, served_requests  # noqa: E402


def quadrant(n, seed):
    """2D Riemann problem: each quadrant draws rho, p ~ U[0.1, 2], u, v ~ U[-1, 1]."""
    rng = np.random.default_rng(seed)
    c = (np.arange(n) + 0.5) / n
    Y, X = np.meshgrid(c, c, indexing="ij")
    q = (X >= 0.5).astype(int) + 2 * (Y >= 0.5).astype(int)
    vals = np.stack([rng.uniform(0.1, 2, 4), rng.uniform(-1, 1, 4), rng.uniform(-1, 1, 4),
                     rng.uniform(0.1, 2, 4)])
    return vals[:, q]


def grids(precision, sizes=(64, 96, 130), limiters=("MINBEE", "Superbee", "VanLeer")):
    return [Grid(quadrant(n, k), [1, 1], precision=precision, t_end=0.2, limiter=lim)
            for k, (n, lim) in enumerate(zip(sizes, limiters))]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batched_equals_alone(precision):
    together = grids(precision)
    alone = grids(precision)
    b = Batch(together, graph_steps=5)
    b.advance(20)
    b.refresh()
    for g in alone:
        s = Batch([g])
        s.advance(20)
        s.refresh()
        s.close()
    for g, h in zip(together, alone):
        assert g.steps == h.steps == 20
        assert g.time == h.time
        np.testing.assert_array_equal(g.state_host(), h.state_host())
    b.close()


def test_rebatching_continues_where_it_stopped():
    gs = grids("fp64")
    ref = grids("fp64")
    b = Batch(gs)
    b.advance(7)
    b.refresh()
    b.close()
    extra = Grid(quadrant(80, 9), [1, 1], precision="fp64", t_end=0.2, limiter="Unos")
    b2 = Batch([gs[2], extra, gs[0]])  # different membership and order
    b2.advance(9)
    b2.refresh()
    for g in ref:
        s = Batch([g])
        s.advance(16 if g is not ref[1] else 7)
        s.refresh()
    for g, h in ((gs[0], ref[0]), (gs[2], ref[2])):
        assert g.steps == h.steps == 16
        assert g.time == h.time
        np.testing.assert_array_equal(g.state_host(), h.state_host())
        np.testing.assert_allclose(g.report.boundary_integral, h.report.boundary_integral,
                                   rtol=1e-12, atol=1e-15)


def test_autotuner_picks_a_configuration_that_runs():
    gs = grids("fp32")
    tile = autotune.tune(gs, steps=2, warmup=1, use_cache=False)
    assert len(tile) == 5
    b = Batch(gs, tile=tile)
    b.advance(3)
    b.refresh()
    assert all(g.steps == 3 for g in gs)


def stream(seed=3):
    reqs = served_requests(rate=200.0, count=10, seed=seed, n1=(1e3, 4e3), n2=(64, 160),
                           n3=(24, 40))
    for r in reqs:
        r.t_end = 0.02
    return reqs


def test_served_results_same_alone_and_in_the_mix():
    """Continuous batching: ten mixed 1D/2D/3D requests arriving at 200/s.
    Each final state equals the same request solved alone, bit for bit."""
    reqs = stream()
    srv = Server(budget_bytes=8 << 30, precision="fp32", steps_per_tick=4, keep_results=True)
    stats = srv.run(reqs)
    assert stats["completed"] == len(reqs)
    assert stats["p99_latency_s"] >= stats["p50_latency_s"] > 0
    assert srv.rebuilds >= 2  # membership changed while others were running
    for r, alone in zip(reqs, stream()):
        g = alone.make_grid("fp32", "cuda")
        b = Batch([g])
        while not g.done:
            b.advance(16)
            b.refresh()
        b.close()
        assert g.steps == r.steps
        np.testing.assert_array_equal(r.result, g.state_host())


def test_admission_waits_for_memory():
    """With a budget the size of the largest request, requests queue and are
    admitted as earlier ones finish; resident bytes never exceed the budget
    and all requests complete."""
    reqs = stream(seed=4)
    for r in reqs:
        r.arrival = 0.0  # all at once: the budget cannot hold them together
    one = max(r.bytes_estimate("fp32") for r in reqs)
    assert sum(r.bytes_estimate("fp32") for r in reqs) > one
    srv = Server(budget_bytes=one, precision="fp32", steps_per_tick=8)
    stats = srv.run(reqs)
    assert stats["completed"] == len(reqs)
    for r in reqs:
        resident = sum(q.bytes_estimate("fp32") for q in reqs
                       if q.admitted <= r.admitted < q.finished)
        assert resident <= one
    first_done = min(r.finished for r in reqs)
    assert any(r.admitted >= first_done for r in reqs)  # someone waited for memory


def blocks3(shape, seed):
    """3D Riemann problem on octants: rho, p ~ U[0.1, 2], velocities ~ U[-1, 1]."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    Z, Y, X = np.meshgrid((np.arange(nz) + 0.5) / nz, (np.arange(ny) + 0.5) / ny,
                          (np.arange(nx) + 0.5) / nx, indexing="ij")
    q = (X >= 0.45).astype(int) + 2 * (Y >= 0.55).astype(int) + 4 * (Z >= 0.5).astype(int)
    vals = np.stack([rng.uniform(0.1, 2, 8)] + [rng.uniform(-1, 1, 8) for _ in range(3)] +
                    [rng.uniform(0.1, 2, 8)])
    return vals[:, q]


@pytest.mark.parametrize("tile", [(16, 12, 40), (16, 12, 7), (32, 8, 40), (24, 8, 16),
                                  (16, 6, 40), (12, 12, 40), (12, 10, 20)])
def test_fp32_3d_state_independent_of_tile_shape(tile):
    """The cell arithmetic does not depend on how cells are dealt to threads:
    the fixed-shape 16x16 and 32x8 kernels, the runtime-shape kernel (16x12,
    24x8, 16x6), tiles whose ring cells run on lanes after the owners (12x12,
    12x10: not whole warps of cells) and short chunks give the same FP32
    state after 12 steps on a grid with partial tiles in x and y, for three
    limiters."""
    shape = (37, 45, 70)
    lims = ("MINBEE", "Superbee", "VanLeer")

    def run(t):
        gs = [Grid(blocks3(shape, 11 + k), [1, 1, 1], precision="fp32", t_end=1.0, limiter=lim)
              for k, lim in enumerate(lims)]
        b = Batch(gs, tile=t)
        b.advance(12)
        b.refresh()
        b.close()
        return gs

    ref = run((16, 16, 40))
    got = run(tile)
    for g, h in zip(got, ref):
        assert g.steps == h.steps == 12
        assert g.time == h.time
        np.testing.assert_array_equal(g.state_host(), h.state_host())


@pytest.mark.parametrize("tile", [(124, 1, 32), (124, 1, 7), (100, 1, 16), (252, 1, 16),
                                  (96, 1, 16), (256, 1, 32)])
def test_fp32_2d_state_independent_of_tile_shape(tile):
    """2D: 128-cell rows (the reference tile here), rows of 124 and 100 cells
    whose two ring cells run on the lanes after the owners, 252 (no tensor
    copies: the box would exceed 256), 96 and 256 give the same FP32 state
    after 12 steps on grids with partial rows, for three limiters."""
    sizes = (250, 190, 131)
    lims = ("MINBEE", "Superbee", "VanLeer")

    def run(t):
        gs = [Grid(quadrant(n, 21 + k), [1, 1], precision="fp32", t_end=1.0, limiter=lim)
              for k, (n, lim) in enumerate(zip(sizes, lims))]
        b = Batch(gs, tile=t)
        b.advance(12)
        b.refresh()
        b.close()
        return gs

    ref = run((128, 1, 32))
    got = run(tile)
    for g, h in zip(got, ref):
        assert g.steps == h.steps == 12
        assert g.time == h.time
        np.testing.assert_array_equal(g.state_host(), h.state_host())
