"""Serving loop for streams of LES solve requests on one GPU.

A request is (grid, roughness length, seed, actuator disks, step count).
Requests of the same grid share *size classes*; a class owns batch handles
("chunks") of a fixed slot capacity, so every kernel of a step advances all
admitted requests of a chunk in one launch, and chunks of different classes
run on their own CUDA streams and overlap on the device.

Admission is continuous: between steps, waiting requests enter free slots of
their class (their fields stay on the device until they finish), and a new
chunk is created only when its device footprint fits the HBM budget.  A
request enters a chunk only at a step that is a multiple of ``cs_count`` of
that chunk, so all its instances share the phase of the dynamic SGS update
and one step in ``cs_count`` carries it.  Finished requests are retired
(mean profiles read back) and their slots reused; empty chunks are freed.

The reference has no serving path (it runs one simulation per MPI job); this
module is host plumbing over the C ABI.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np


@dataclass
class Request:
    rid: int
    grid: Tuple[int, int, int]           # (nx, ny, Nz)
    zo: float
    seed: int
    steps: int
    turbines: List[dict] = field(default_factory=list)
    arrival: float = 0.0                 # seconds after the stream start
    # filled by the server
    admitted: Optional[float] = None
    finished: Optional[float] = None
    result: Optional[dict] = None

    @property
    def points(self) -> int:
        nx, ny, nz = self.grid
        return nx * ny * nz


class GpuBackend:
    """Batch handles of the CUDA library."""

    def __init__(self, precision: str = "mixed", **base):
        self.precision = precision
        self.base = base

    def slot_bytes(self, grid) -> int:
        from .solver import footprint_bytes
        nx, ny, nz = grid
        return footprint_bytes(1, nx=nx, ny=ny, Nz=nz, precision=self.precision, **self.base)

    def create(self, grid, capacity):
        from .solver import LesgoBatch
        nx, ny, nz = grid
        return LesgoBatch(capacity, nx=nx, ny=ny, Nz=nz, precision=self.precision, **self.base)

    @staticmethod
    def add(h, req: Request) -> int:
        return h.add(req.zo, req.seed, req.turbines)

    @staticmethod
    def step(h):
        h.step(1)          # asynchronous on the handle's stream

    @staticmethod
    def sync(h):
        h.sync()

    @staticmethod
    def collect(h, iid: int, req: Request) -> dict:
        u = h.get(iid, "u")
        nz = h.nz
        prof = u[1:nz, :, :h.nx].mean(axis=(1, 2))
        out = dict(u_profile=prof, diag=h.diag(iid))
        if req.turbines:
            out["power"] = h.turbine_state(iid)["power"]
        return out

    @staticmethod
    def remove(h, iid: int):
        h.remove(iid)

    @staticmethod
    def close(h):
        h.close()


@dataclass
class Chunk:
    handle: object
    capacity: int
    nbytes: int
    step: int = 0
    members: Dict[int, Tuple[Request, int]] = field(default_factory=dict)   # iid -> (request, steps done)


class Server:
    def __init__(self, backend, budget_bytes: float = 150e9, chunk_slots: int = 8, cs_count: int = 5,
                 clock: Callable[[], float] = time.perf_counter):
        self.backend = backend
        self.budget = budget_bytes
        self.chunk_slots = chunk_slots
        self.cs_count = cs_count
        self.clock = clock
        self.classes: Dict[Tuple[int, int, int], List[Chunk]] = {}
        self.waiting: List[Request] = []
        self.done: List[Request] = []
        self.allocated = 0
        self.point_steps = 0
        self.steps_issued = 0
        self._slot_bytes: Dict[Tuple[int, int, int], int] = {}

    # ---------------- admission --------------------------------------------------
    def slot_bytes(self, grid) -> int:
        if grid not in self._slot_bytes:
            self._slot_bytes[grid] = self.backend.slot_bytes(grid)
        return self._slot_bytes[grid]

    def submit(self, req: Request):
        self.waiting.append(req)

    def _admit(self, now: float):
        still = []
        for req in self.waiting:
            if req.arrival > now:
                still.append(req)
                continue
            if not self._place(req, now):
                still.append(req)
        self.waiting = still

    def _place(self, req: Request, now: float) -> bool:
        chunks = self.classes.setdefault(req.grid, [])
        for ch in chunks:
            # an empty chunk has no phase to keep; a busy one admits at its SGS phase
            if len(ch.members) < ch.capacity and (not ch.members or ch.step % self.cs_count == 0):
                if not ch.members:
                    ch.step = 0
                iid = self.backend.add(ch.handle, req)
                ch.members[iid] = (req, 0)
                req.admitted = now
                return True
        if any(len(ch.members) < ch.capacity for ch in chunks):
            return False              # a slot frees up at the chunk's next SGS phase
        nbytes = self.slot_bytes(req.grid) * self.chunk_slots
        if nbytes > self.budget:
            raise ValueError(f"a chunk of grid {req.grid} ({nbytes} B) exceeds the HBM budget")
        if self.allocated + nbytes > self.budget:
            return False              # waits for memory
        h = self.backend.create(req.grid, self.chunk_slots)
        ch = Chunk(h, self.chunk_slots, nbytes)
        chunks.append(ch)
        self.allocated += nbytes
        iid = self.backend.add(h, req)
        ch.members[iid] = (req, 0)
        req.admitted = now
        return True

    # ---------------- stepping ----------------------------------------------------
    def _tick(self):
        active = [ch for chs in self.classes.values() for ch in chs if ch.members]
        for ch in active:                 # launch every chunk first: they overlap on the GPU
            self.backend.step(ch.handle)
        for ch in active:
            self.backend.sync(ch.handle)
        now = self.clock() - self.t0
        for ch in active:
            ch.step += 1
            finished = []
            for iid, (req, n) in ch.members.items():
                n += 1
                ch.members[iid] = (req, n)
                self.point_steps += req.points
                if n >= req.steps:
                    finished.append(iid)
            for iid in finished:
                req, _ = ch.members.pop(iid)
                req.result = self.backend.collect(ch.handle, iid, req)
                self.backend.remove(ch.handle, iid)
                req.finished = now
                self.done.append(req)
        self.steps_issued += 1
        # free chunks that stay empty
        for grid, chs in self.classes.items():
            keep = []
            for ch in chs:
                if not ch.members and not any(r.grid == grid and r.arrival <= now for r in self.waiting):
                    self.backend.close(ch.handle)
                    self.allocated -= ch.nbytes
                else:
                    keep.append(ch)
            self.classes[grid] = keep

    def run(self, requests: List[Request], idle_sleep: float = 0.0005) -> dict:
        for r in sorted(requests, key=lambda r: r.arrival):
            self.submit(r)
        self.t0 = self.clock()
        busy = 0.0
        while self.waiting or any(ch.members for chs in self.classes.values() for ch in chs):
            now = self.clock() - self.t0
            self._admit(now)
            if any(ch.members for chs in self.classes.values() for ch in chs):
                t = self.clock()
                self._tick()
                busy += self.clock() - t
            elif self.waiting:
                nxt = min(r.arrival for r in self.waiting)
                wait = nxt - (self.clock() - self.t0)
                if wait > 0:
                    time.sleep(min(wait, idle_sleep if idle_sleep > 0 else wait))
        wall = self.clock() - self.t0
        return self.report(wall, busy)

    def report(self, wall: float, busy: float) -> dict:
        lat = np.array([r.finished - r.arrival for r in self.done]) if self.done else np.zeros(1)
        return dict(requests=len(self.done), wall_s=wall, busy_frac=busy / wall if wall > 0 else 0.0,
                    point_steps=self.point_steps, throughput=self.point_steps / wall if wall > 0 else 0.0,
                    p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)),
                    max_allocated_bytes=self.allocated)


def poisson_requests(n: int, rate: float, grids, steps_range, seed: int = 0, turbines_max: int = 0,
                     zo_range=(1e-5, 1e-3)) -> List[Request]:
    """Seeded request stream: Poisson arrivals, grid from `grids`, z0
    log-uniform, 0..turbines_max actuator disks (D = 0.1, Ct' = 1.33, hub
    0.1, non-overlapping on a 7D x 5D lattice), steps uniform in steps_range."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    lo, hi = math.log(zo_range[0]), math.log(zo_range[1])
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        grid = tuple(grids[rng.integers(len(grids))])
        nt = int(rng.integers(turbines_max + 1)) if turbines_max > 0 else 0
        lattice = [(0.5 + 0.7 * a, 0.4 + 0.5 * b) for a in range(8) for b in range(6)]
        picks = rng.permutation(len(lattice))[:nt]
        tb = [dict(xloc=lattice[p][0], yloc=lattice[p][1], height=0.1, dia=0.1, thk=0.001, Ct_prime=1.33)
              for p in picks]
        out.append(Request(rid=i, grid=grid, zo=math.exp(rng.uniform(lo, hi)), seed=1000 + i,
                           steps=int(rng.integers(steps_range[0], steps_range[1] + 1)), turbines=tb, arrival=t))
    return out
