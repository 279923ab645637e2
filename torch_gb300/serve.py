"""Continuous-batching request server for mixed 1D/2D/3D solves on one GPU.

Requests arrive over time; each asks for one Cartesian solve to its t_end.
The server loop admits arrived requests while their device memory fits the
HBM budget, keeps every admitted grid resident until it completes, and
advances all resident grids of one dimension together with one launch per
stage (``batch.Batch``), each dimension on its own CUDA stream so that 1D,
2D and 3D work overlaps.  Grids that finish leave their batch and free their
memory; waiting requests join when their dimension's batch next goes idle.  Results of a
grid are the same alone and in the mix: every grid keeps its own dt and the
per-cell arithmetic does not depend on what else is resident.

TORCH has no serving layer; the request workload follows the served-stream
configuration (Poisson arrivals, 40% 1D Sod tubes, 40% 2D and 20% 3D
explosions, random states, t_end in [0.1, 0.3]).
"""

import math
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from .batch import Batch, Grid


@dataclass
class Request:
    rid: int
    dim: int
    n: int
    arrival: float                 # seconds after the stream starts
    t_end: float
    limiter: str
    inside: tuple                  # (rho, p) inside / left
    outside: tuple                 # (rho, p) outside / right
    admitted: Optional[float] = None
    finished: Optional[float] = None
    steps: int = 0
    status: int = -1
    cells: int = 0
    grid: Optional[Grid] = field(default=None, repr=False)
    result: Optional[np.ndarray] = field(default=None, repr=False)  # final state (host)

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival

    def primitive(self):
        """Initial primitives: 1D Sod-type tube split at 1/2; 2D disc / 3D
        sphere of radius 0.2 at the centre of the unit box."""
        n, d = self.n, self.dim
        c = (np.arange(n) + 0.5) / n
        if d == 1:
            left = c < 0.5
            p = np.zeros((3, n))
            p[0] = np.where(left, self.inside[0], self.outside[0])
            p[2] = np.where(left, self.inside[1], self.outside[1])
            return p
        mesh = np.meshgrid(*([c] * d), indexing="ij")
        inside = sum((m - 0.5) ** 2 for m in mesh) <= 0.2 ** 2
        p = np.zeros((d + 2,) + (n,) * d)
        p[0] = np.where(inside, self.inside[0], self.outside[0])
        p[-1] = np.where(inside, self.inside[1], self.outside[1])
        return p

    def make_grid(self, precision, device):
        return Grid(self.primitive(), [1.0] * self.dim, precision=precision, device=device,
                    t_end=self.t_end, cfl=0.4, limiter=self.limiter,
                    boundaries=["Open"] * self.dim, tag=self.rid)

    def bytes_estimate(self, precision):
        per = (8 if precision == "fp64" else 4) * self.n ** self.dim
        # state ring of two buffers plus the batch workspace share (per-tile partials)
        return 2 * (self.dim + 2) * per + per // 8 + 4096


def served_requests(rate, count, seed=0, n1=(1e3, 1e5), n2=(128, 1024), n3=(64, 256)):
    """The served-stream workload: Poisson arrivals at `rate` requests/s."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(count):
        t += rng.exponential(1.0 / rate)
        u = rng.random()
        if u < 0.4:
            dim, n = 1, int(round(10 ** rng.uniform(math.log10(n1[0]), math.log10(n1[1]))))
        elif u < 0.8:
            dim, n = 2, int(rng.integers(n2[0], n2[1] + 1))
        else:
            dim, n = 3, int(rng.integers(n3[0], n3[1] + 1))
        inside = (float(rng.uniform(0.1, 2.0)), float(rng.uniform(0.1, 2.0)))
        outside = (float(rng.uniform(0.1, 2.0)), float(rng.uniform(0.1, 2.0)))
        out.append(Request(rid, dim, n, t, float(rng.uniform(0.1, 0.3)),
                           "VanLeer" if rng.random() < 0.5 else "Superbee", inside, outside))
    return out


class Server:
    """Admit, batch and advance requests until all are done.

    One batch per dimension, each on its own CUDA stream.  The host loop polls
    the batches: a batch whose enqueued steps are done is refreshed, loses its
    finished grids and gains newly admitted ones (a rebuild), and is given its
    next slice of steps.  Slices are sized per batch from its measured step
    time so that each slice takes about `slice_ms` on the device: a batch of
    small 1D tubes takes hundreds of steps per slice while a batch holding a
    256^3 grid takes one or two, and neither waits for the other.
    """

    def __init__(self, budget_bytes, precision="fp32", steps_per_tick=8, tile=None,
                 device=None, max_resident=256, clock=time.perf_counter, keep_results=False,
                 graphs=True, slice_ms=2.0, max_slice=512):
        self.keep_results = keep_results
        self.graphs = graphs  # each batch replays a captured graph of `steps_per_tick` steps
        self.budget = int(budget_bytes)
        self.precision = precision
        self.k = int(steps_per_tick)
        self.slice_ms = float(slice_ms)
        self.max_slice = int(max_slice)
        self.tiles = tile or {}
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.max_resident = max_resident
        self.clock = clock
        self.used = 0
        self.resident = {1: [], 2: [], 3: []}
        self.batches = {}
        self.slice = {1: self.k, 2: self.k, 3: self.k}
        self.streams = {d: torch.cuda.Stream(self.device) for d in (1, 2, 3)}
        self.ticks = 0
        self.rebuilds = 0

    def _keep(self, r):
        """keep_results: True keeps every final state on the host, a set of
        request ids keeps those requests' states only."""
        k = self.keep_results
        return k is True or (bool(k) and not isinstance(k, bool) and r.rid in k)

    def _rebuild(self, dim):
        old = self.batches.pop(dim, None)
        if old is not None:
            old.close()
        grids = [r.grid for r in self.resident[dim]]
        if grids:
            self.batches[dim] = Batch(grids, tile=self.tiles.get(dim), stream=self.streams[dim],
                                      graph_steps=self.k if self.graphs else 0)
            self.rebuilds += 1

    def _retire(self, dim, t0):
        """Refresh an idle batch; finished grids leave.  True if any left."""
        b = self.batches[dim]
        timing = b.last_ms()
        if timing is not None and timing[0] > 0:
            per_step = timing[0] / timing[1]
            self.slice[dim] = max(1, min(self.max_slice, int(self.slice_ms / per_step)))
        b.refresh()
        still, left = [], False
        for r in self.resident[dim]:
            if r.grid.done:
                r.finished = self.clock() - t0
                r.steps = r.grid.steps
                r.status = r.grid.status
                if self._keep(r):
                    r.result = r.grid.state_host()
                self.used -= r.bytes_estimate(self.precision)
                r.grid = None
                left = True
            else:
                still.append(r)
        self.resident[dim] = still
        return left

    def run(self, requests: List[Request]):
        pending = sorted(requests, key=lambda r: r.arrival)
        waiting = []
        dirty = set()  # dimensions whose membership changed since their batch was built
        t0 = self.clock()
        i = 0
        while i < len(pending) or waiting or any(self.resident.values()):
            now = self.clock() - t0
            while i < len(pending) and pending[i].arrival <= now:
                waiting.append(pending[i])
                i += 1
            keep = []
            for r in waiting:  # admission in arrival order while memory allows
                need = r.bytes_estimate(self.precision)
                nres = sum(len(v) for v in self.resident.values())
                if self.used + need <= self.budget and nres < self.max_resident:
                    r.grid = r.make_grid(self.precision, self.device)
                    r.cells = r.grid.cells
                    r.admitted = self.clock() - t0
                    self.used += need
                    self.resident[r.dim].append(r)
                    dirty.add(r.dim)
                else:
                    keep.append(r)
            waiting = keep
            issued = False
            for d in (1, 2, 3):
                b = self.batches.get(d)
                if b is not None:
                    if not b.idle():
                        continue
                    if self._retire(d, t0):
                        dirty.add(d)
                if d in dirty:
                    self._rebuild(d)
                    dirty.discard(d)
                b = self.batches.get(d)
                if b is not None and not b.all_done():
                    b.advance_async(self.slice[d])
                    issued = True
            if issued:
                self.ticks += 1
            elif i < len(pending) and not any(self.resident.values()) and not waiting:
                time.sleep(max(0.0, min(0.01, pending[i].arrival - (self.clock() - t0))))
            else:
                time.sleep(5e-5)
        for b in self.batches.values():
            b.close()
        self.batches = {}
        return summarize(requests, self.clock() - t0)


def summarize(requests, wall):
    lat = np.array([r.latency for r in requests if r.latency is not None])
    cu = sum(r.cells * r.steps for r in requests)
    return {
        "requests": len(requests),
        "completed": int(sum(r.status == 1 for r in requests)),
        "wall_s": wall,
        "cell_updates": cu,
        "cell_updates_per_s": cu / wall if wall > 0 else None,
        "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
    }
