"""Serving loop: a stream of solve requests over a catalogue of systems.

Each request names a system, a 3D 7-point Dirichlet Laplacian or the tet-cube
biharmonic smoothing system ``alpha M + K M^-1 K`` of a given grid side, and
carries k <= 8 right-hand sides.  The server keeps each system's operator,
FSAI factor and Krylov state resident in device memory under a byte budget
(least recently used idle systems are evicted to admit new ones; a system
that cannot fit at all is rejected) and runs requests in slots, one CUDA
stream each.  A free slot takes the oldest queued request whose system is
idle, copies its right-hand sides in, runs the whole PCG loop as one CUDA
graph (k > 1: the batched solver, which reads the matrices once per
iteration for all k right-hand sides; k = 1: the single-vector solver, which
runs a small system's whole solve as one kernel on a thread-block cluster;
with ``GpuExecutor(cluster_rhs=True)`` a small system's k > 1 right-hand
sides also run that way, one cluster each in one launch),
copies x back, and is free for the next request as soon as its event fires.
Requests join and leave the running set one by one, so none waits for a
batch to fill or for an unrelated long solve.

A system has at most one solve in flight (its operators own their scratch
vectors); requests for a busy system wait while others go ahead.  Results do
not depend on what else runs: every kernel's reduction order is fixed by the
system size and k, so a request gives bit-identical x alone and in the mix.

``GpuExecutor(merge_rhs=m)`` also merges queued requests for one system:
when a slot takes a request, later queued requests for the same system join
it while their right-hand sides fit in m, and the group runs as one batched
solve (each right-hand side its own CG recurrence, the matrices read once
per iteration for all of them).  A merged request's x then equals its
unmerged solve to the solve tolerance, not bit for bit (the batched dot
products fold over the group's width).

``GpuExecutor(sequential=True)`` is the plain one-at-a-time float64 path for
comparison: one slot, and the k right-hand sides of a request solved one
after another with the single-vector solver.

The scheduler (``Server``) only talks to an executor through ``estimate``,
``build``, ``release``, ``start``, ``poll`` and ``finish``, so its admission,
eviction and failure handling run on the CPU with a stand-in executor.
"""

from __future__ import annotations

import collections
import math
import queue
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import Callable

import numpy as np
import torch

ALPHA = 1.0e-4  # mass weight of the biharmonic smoothing systems
KINDS = ("laplacian", "biharmonic")
MAX_RHS = 8


# ---------------------------------------------------------------------------
# Requests.

@dataclass(frozen=True)
class Request:
    rid: int
    kind: str
    side: int
    k: int
    arrival: float  # seconds after the start of the stream
    seed: int

    @property
    def key(self) -> tuple[str, int]:
        return (self.kind, self.side)

    @property
    def n(self) -> int:
        return self.side ** 3


def request_stream(count: int = 2000, rate: float = 4.0, seed: int = 0, n_min: float = 5e3,
                   n_max: float = 5e5, k_max: int = MAX_RHS, kinds=KINDS) -> list[Request]:
    """Seeded request stream: kind uniform over `kinds`; n log-uniform on
    [n_min, n_max], mapped to the nearest grid side (n = side^3 unknowns for
    both kinds); k uniform on 1..k_max; Poisson arrivals at `rate` per second."""
    if count < 0 or rate <= 0 or not 0 < n_min <= n_max or not 1 <= k_max <= MAX_RHS:
        raise ValueError("request_stream: bad arguments")
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=count))
    kind_idx = rng.integers(0, len(kinds), size=count)
    n = np.exp(rng.uniform(math.log(n_min), math.log(n_max), size=count))
    sides = np.maximum(3, np.rint(np.cbrt(n))).astype(int)
    ks = rng.integers(1, k_max + 1, size=count)
    seeds = rng.integers(0, 2**31 - 1, size=count)
    return [Request(i, kinds[int(kind_idx[i])], int(sides[i]), int(ks[i]), float(arrivals[i]),
                    int(seeds[i])) for i in range(count)]


def request_rhs(req: Request, pin: bool = False) -> torch.Tensor:
    """The request's right-hand sides: [n, k] float64, uniform on [-1, 1], seeded."""
    data = np.random.default_rng(req.seed).uniform(-1.0, 1.0, size=(req.n, req.k))
    t = torch.from_numpy(data)
    return t.pin_memory() if pin else t


@dataclass
class Result:
    rid: int
    key: tuple[str, int]
    k: int
    arrival: float
    start: float = math.nan
    done: float = math.nan
    x: torch.Tensor | None = None  # [n, k] float64 (host)
    iterations: list[int] | None = None
    error: str | None = None

    @property
    def latency(self) -> float:
        return self.done - self.arrival

    @property
    def ok(self) -> bool:
        return self.error is None


class Rejected(Exception):
    """A request that can never be admitted (its system exceeds the budget)."""


# ---------------------------------------------------------------------------
# Host systems.

@dataclass
class HostSystem:
    kind: str
    side: int
    n: int
    A: object                # scipy CSR: the Laplacian L, or the stiffness K
    mass: np.ndarray | None  # lumped mass (biharmonic)

    def assembled(self):
        """The matrix the FSAI factor approximates, assembled on the host: L,
        or Q = alpha M + K M^-1 K.  Only for checking: resident systems
        assemble Q on the device."""
        if self.kind == "laplacian":
            return self.A
        from . import problems

        return problems.biharmonic(self.A, self.mass, ALPHA)


def host_system(kind: str, side: int) -> HostSystem:
    from . import problems

    if kind == "laplacian":
        L = problems.laplacian_3d(side)
        return HostSystem(kind, side, L.shape[0], L, None)
    if kind == "biharmonic":
        _, _, K, mass = problems.tet_cube(side)
        return HostSystem(kind, side, K.shape[0], K, mass)
    raise ValueError(f"unknown system kind {kind!r}")


class Catalog:
    """Host-assembled systems by (kind, side), built on first use."""

    def __init__(self, builder: Callable[[str, int], HostSystem] = host_system):
        self._builder = builder
        self._systems: dict[tuple[str, int], HostSystem] = {}
        self._lock = threading.Lock()

    def get(self, key) -> HostSystem:
        with self._lock:
            s = self._systems.get(key)
        if s is None:
            s = self._builder(*key)
            with self._lock:
                self._systems.setdefault(key, s)
        return s

    def prebuild(self, keys, threads: int = 8) -> None:
        """Assemble several systems at once (numpy and SciPy release the GIL)."""
        todo = sorted(set(keys), key=lambda k: -k[1])
        with ThreadPoolExecutor(max(1, threads)) as ex:
            list(ex.map(self.get, todo))

    def __contains__(self, key) -> bool:
        return key in self._systems


def estimate_bytes(host: HostSystem, max_rhs: int = MAX_RHS, width: int = 8) -> int:
    """Upper bound on the device bytes of a resident system (operators in
    sliced-ELL and CSR form, FSAI factor and transpose in both forms, Krylov
    state for one and for max_rhs right-hand sides)."""
    n, nnz = host.n, host.A.nnz
    nnz_g = width * n  # rows of G hold at most `width` entries
    csr = lambda e: 12 * e + 4 * (n + 1)
    sell = lambda e: int(1.5 * 12 * e) + 8 * n
    vec, blk = 8 * n, 8 * n * max_rhs
    a_copies = 1 if host.kind == "laplacian" else 2
    single = csr(nnz) + a_copies * sell(nnz) + 4 * vec  # torch CSR + product matrices + scratch
    single += 2 * csr(nnz_g) + 2 * sell(nnz_g) + 2 * vec  # G, GT (torch and sliced ELL) + scale
    single += 8 * vec + 4 * n  # Krylov state, b/x, free indices
    batched = a_copies * csr(nnz) + 2 * csr(nnz_g) + 2 * blk  # matrices + operator scratch
    batched += 6 * blk  # Krylov state, B and X
    return int(1.25 * (single + batched)) + (4 << 20)


# ---------------------------------------------------------------------------
# Device side.

class ResidentSystem:
    """Device-resident operator, FSAI factor and Krylov state of one system."""

    def __init__(self, host: HostSystem, *, width: int = 8, step: int = 1, kap: float = 1e-3,
                 max_rhs: int = MAX_RHS, batched: bool = True, cluster_rhs: bool = False,
                 device="cuda"):
        from .batched import BatchedCG, batched_fsai, batched_sparse, batched_sqlap
        from .fsai import FSAI
        from .linear import Solver, aslinearoperator
        from .sparse import from_scipy, spgemm
        from .squared_laplacian import SquaredLaplacianOperator

        dev = torch.device(device)
        self.key = (host.kind, host.side)
        self.n = n = host.n
        self.max_rhs = max_rhs
        A = from_scipy(host.A, dev)
        if host.kind == "laplacian":
            P = A
        else:
            # Q = K diag(1 / m) K + diag(alpha m) by the device SpGEMM, equal
            # bit for bit to the host SciPy assembly.
            mass = torch.as_tensor(host.mass, dtype=torch.float64, device=dev)
            P = spgemm(A, A, col_scale=1.0 / mass, add_diag=ALPHA * mass)
        self.fsai = FSAI(P, max_row_size=width, kap_tolerance=kap, max_step_size=step)
        self.fsai.source = None  # the solves need only the factor
        del P
        if host.kind == "laplacian":
            self.A = aslinearoperator(A)
        else:
            free = torch.arange(n, dtype=torch.int32, device=dev)
            self.A = SquaredLaplacianOperator(A, mass, free, mass_weight=ALPHA)
        self.solver = Solver("cg", self.A, self.fsai)
        self.b1 = torch.zeros(n, dtype=torch.float64, device=dev)
        self.x1 = torch.zeros(n, dtype=torch.float64, device=dev)
        self.nit = torch.zeros(max_rhs, dtype=torch.int32, device=dev)
        self.B = torch.zeros(n * max_rhs, dtype=torch.float64, device=dev)
        self.X = torch.zeros(n * max_rhs, dtype=torch.float64, device=dev)
        self.bcg = None
        self.csolver = None
        if batched and cluster_rhs and max_rhs > 1 and self.solver.cluster_size > 0:
            # A small system: its single-vector solve runs on one thread-block
            # cluster, so the k right-hand sides of a request run as k such
            # solves in one launch, each the single-vector result bit for bit.
            from .multi import ClusterSolver

            self.csolver = ClusterSolver([(self.A, self.fsai)] * max_rhs)
            self.BT = torch.zeros((max_rhs, n), dtype=torch.float64, device=dev)
            self.XT = torch.zeros((max_rhs, n), dtype=torch.float64, device=dev)
        elif batched and max_rhs > 1:
            if host.kind == "laplacian":
                BA = batched_sparse(A)
            else:
                BA = batched_sqlap(A, self.A.mass, ALPHA, torch.float64, torch.float64,
                                   max_rhs=max_rhs)
            BM = batched_fsai(self.fsai, torch.float64, torch.float64, max_rhs=max_rhs)
            self.bcg = BatchedCG(BA, BM, max_rhs=max_rhs)

    def warm(self, tol: float) -> None:
        """Capture every solver graph the serving loop will launch (one
        iteration each), so that no capture happens while requests wait."""
        self.solver.run(self.b1, self.x1, tol, 0.0, 1)
        if self.bcg is not None:
            for k in range(2, self.max_rhs + 1):
                B, X = self._blocks(k)
                self.bcg.run(B, X, tol, 0.0, 1)

    def _blocks(self, k):
        n = self.n
        return self.B[: n * k].view(n, k), self.X[: n * k].view(n, k)

    def launch(self, rhs: torch.Tensor, out: torch.Tensor, nit_out: torch.Tensor,
               stream: torch.cuda.Stream, sequential: bool, tol: float, maxiter: int):
        """Enqueue one request on `stream`: copy in, solve, copy x and the
        iteration counts out; returns the event that marks completion."""
        n, k = rhs.shape
        if n != self.n or not 1 <= k <= self.max_rhs:
            raise ValueError(f"right-hand sides of shape {tuple(rhs.shape)} do not fit system "
                             f"{self.key} (n={self.n}, k <= {self.max_rhs})")
        with torch.cuda.stream(stream):
            if k == 1:
                self.b1.copy_(rhs.view(-1), non_blocking=True)
                self.x1.zero_()
                nit, _, _ = self.solver.run(self.b1, self.x1, tol, 0.0, maxiter)
                out.view(-1).copy_(self.x1, non_blocking=True)
                nit_out.copy_(nit, non_blocking=True)
            elif self.csolver is not None and not sequential:
                self.BT[:k].copy_(rhs.to(self.BT.device, non_blocking=True).t())
                self.XT[:k].zero_()
                nit, _, _ = self.csolver.run(list(self.BT[:k]), list(self.XT[:k]), tol, 0.0,
                                             maxiter)
                out.copy_(self.XT[:k].t(), non_blocking=True)
                nit_out.copy_(nit, non_blocking=True)
            elif sequential or self.bcg is None:
                B, X = self._blocks(k)
                B.copy_(rhs, non_blocking=True)
                for j in range(k):
                    self.b1.copy_(B[:, j])
                    self.x1.zero_()
                    nit, _, _ = self.solver.run(self.b1, self.x1, tol, 0.0, maxiter)
                    X[:, j].copy_(self.x1)
                    self.nit[j:j + 1].copy_(nit)
                out.copy_(X, non_blocking=True)
                nit_out.copy_(self.nit[:k], non_blocking=True)
            else:
                B, X = self._blocks(k)
                B.copy_(rhs, non_blocking=True)
                X.zero_()
                nit, _ = self.bcg.run(B, X, tol, 0.0, maxiter)
                out.copy_(X, non_blocking=True)
                nit_out.copy_(nit, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return ev

    def launch_group(self, rhss, outs, nit_out: torch.Tensor, stream: torch.cuda.Stream,
                     tol: float, maxiter: int):
        """Several requests for this system as one batched solve: their
        right-hand sides side by side in one [n, k] block (k = their sum <=
        max_rhs), each column its own CG recurrence; x and the iteration
        counts go back to each request's buffers."""
        ks = [int(r.shape[1]) for r in rhss]
        k = sum(ks)
        if len(rhss) == 1 or k == 1 or (self.bcg is None and self.csolver is None):
            raise ValueError("launch_group takes two or more requests on a batched system")
        if k > self.max_rhs or any(int(r.shape[0]) != self.n for r in rhss):
            raise ValueError(f"request group of {k} right-hand sides does not fit system "
                             f"{self.key} (n={self.n}, k <= {self.max_rhs})")
        if self.csolver is not None:
            with torch.cuda.stream(stream):
                c = 0
                for rhs, kk in zip(rhss, ks):
                    self.BT[c:c + kk].copy_(rhs.to(self.BT.device, non_blocking=True).t())
                    c += kk
                self.XT[:k].zero_()
                nit, _, _ = self.csolver.run(list(self.BT[:k]), list(self.XT[:k]), tol, 0.0,
                                             maxiter)
                c = 0
                for out, kk in zip(outs, ks):
                    out.copy_(self.XT[c:c + kk].t(), non_blocking=True)
                    c += kk
                nit_out.copy_(nit, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(stream)
            return ev
        with torch.cuda.stream(stream):
            B, X = self._blocks(k)
            c = 0
            for rhs, kk in zip(rhss, ks):
                B[:, c:c + kk].copy_(rhs.to(B.device, non_blocking=True))
                c += kk
            X.zero_()
            nit, _ = self.bcg.run(B, X, tol, 0.0, maxiter)
            c = 0
            for out, kk in zip(outs, ks):
                out.copy_(X[:, c:c + kk], non_blocking=True)
                c += kk
            nit_out.copy_(nit[:k], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return ev


class GpuExecutor:
    """Resident systems and slots (CUDA streams) on one GPU."""

    def __init__(self, catalog: Catalog, *, slots: int = 16, sequential: bool = False,
                 tol: float = 1e-8, maxiter: int = 0, width: int = 8, step: int = 1,
                 kap: float = 1e-3, max_rhs: int = MAX_RHS, merge_rhs: int = 0,
                 cluster_rhs: bool = False, wide_from: int = 0, wide_width: int = 48,
                 wide_step: int = 2, device="cuda"):
        if not torch.cuda.is_available():
            raise RuntimeError("GpuExecutor needs a CUDA device")
        if merge_rhs and not 2 <= merge_rhs <= 32:
            raise ValueError("merge_rhs must be 0 (off) or in [2, 32]")
        self.catalog = catalog
        self.sequential = sequential
        self.slots = 1 if sequential else int(slots)
        self.tol, self.maxiter = float(tol), int(maxiter)
        self.width, self.step, self.kap = width, step, kap
        # Queued requests for one system are merged into batched solves of up
        # to merge_rhs right-hand sides (0: one request per solve).
        self.merge_rhs = 0 if sequential else int(merge_rhs)
        self.max_rhs = max(max_rhs, self.merge_rhs)
        # cluster_rhs: a small system runs a request's k right-hand sides as k
        # cluster solves in one launch, instead of the batched solver.
        self.cluster_rhs = bool(cluster_rhs)
        # wide_from > 0: systems of at least that many unknowns get an FSAI
        # factor of width wide_width grown wide_step entries at a time (fewer
        # iterations for a longer setup, paid once while the system is
        # resident).
        self.wide_from, self.wide_width, self.wide_step = (int(wide_from), int(wide_width),
                                                           int(wide_step))
        self.device = torch.device(device)
        self.streams = [torch.cuda.Stream(self.device) for _ in range(self.slots)]

    def _wide(self, host: HostSystem) -> bool:
        return self.wide_from > 0 and host.n >= self.wide_from

    def width_for(self, host: HostSystem) -> int:
        return self.wide_width if self._wide(host) else self.width

    def estimate(self, key) -> int:
        host = self.catalog.get(key)
        return estimate_bytes(host, self.max_rhs, self.width_for(host))

    def build(self, key):
        from . import _lib

        host = self.catalog.get(key)
        cur = torch.cuda.current_stream(self.device)
        cur.synchronize()
        m0, l0 = torch.cuda.memory_allocated(self.device), _lib.live_device_bytes()
        res = ResidentSystem(host, width=self.width_for(host),
                             step=self.wide_step if self._wide(host) else self.step, kap=self.kap,
                             max_rhs=self.max_rhs, batched=not self.sequential,
                             cluster_rhs=self.cluster_rhs, device=self.device)
        res.warm(self.tol)
        cur.synchronize()
        nbytes = (torch.cuda.memory_allocated(self.device) - m0) + (_lib.live_device_bytes() - l0)
        return res, int(nbytes)

    def release(self, handle: ResidentSystem) -> None:
        del handle  # library objects synchronise the device and free on collection

    def start(self, slot: int, handle: ResidentSystem, req: Request, rhs: torch.Tensor):
        out = torch.empty((req.n, req.k), dtype=torch.float64, pin_memory=True)
        nit = torch.empty(req.k, dtype=torch.int32, pin_memory=True)
        ev = handle.launch(rhs, out, nit, self.streams[slot], self.sequential, self.tol,
                           self.maxiter)
        return (ev, out, nit, rhs)

    def start_group(self, slot: int, handle: ResidentSystem, reqs, rhss):
        outs = [torch.empty((r.n, r.k), dtype=torch.float64, pin_memory=True) for r in reqs]
        nit = torch.empty(sum(r.k for r in reqs), dtype=torch.int32, pin_memory=True)
        ev = handle.launch_group(rhss, outs, nit, self.streams[slot], self.tol, self.maxiter)
        return (ev, outs, nit, rhss, [r.k for r in reqs])

    def poll(self, token) -> bool:
        return token[0].query()

    def finish(self, token):
        token[0].synchronize()
        return token[1], [int(v) for v in token[2]]

    def finish_group(self, token):
        """(x, iterations) of each request of a group started by start_group."""
        token[0].synchronize()
        its = [int(v) for v in token[2]]
        out, c = [], 0
        for x, k in zip(token[1], token[4]):
            out.append((x, its[c:c + k]))
            c += k
        return out


# ---------------------------------------------------------------------------
# Scheduler.

class Server:
    """Admission under a device-byte budget, LRU residency and slot dispatch.

    ``run(requests)`` replays a request stream in real time: a producer
    thread hands each request over at its arrival time (with its right-hand
    sides from `make_rhs`), and the calling thread dispatches, polls and
    collects.  Failures of the producer are reported per request; a producer
    that stops altogether fails the requests it never sent.
    """

    def __init__(self, executor, budget_bytes: float = 120e9, idle_sleep: float = 50e-6):
        self.ex = executor
        self.budget = int(budget_bytes)
        self.idle_sleep = idle_sleep
        self.resident: collections.OrderedDict = collections.OrderedDict()  # key -> [handle, bytes]
        self.used = 0
        self.peak = 0
        self.busy: set = set()
        self.stats = dict(builds=0, evictions=0, rejected=0, build_s=0.0, failed=0)

    # -- residency --------------------------------------------------------
    def _make_room(self, need: int) -> bool:
        for key in list(self.resident):  # least recently used first
            if self.used + need <= self.budget:
                break
            if key in self.busy:
                continue
            handle, nbytes = self.resident.pop(key)
            self.ex.release(handle)
            self.used -= nbytes
            self.stats["evictions"] += 1
        return self.used + need <= self.budget

    def ensure(self, key):
        """The resident handle of `key`, building it if needed; None while
        there is no room yet (busy systems hold it).  Raises Rejected when the
        system cannot fit in the budget at all."""
        entry = self.resident.get(key)
        if entry is not None:
            self.resident.move_to_end(key)
            return entry[0]
        est = int(self.ex.estimate(key))
        if est > self.budget:
            raise Rejected(f"system {key} needs about {est} device bytes, more than the "
                           f"{self.budget}-byte budget")
        if not self._make_room(est):
            return None
        t = time.perf_counter()
        handle, nbytes = self.ex.build(key)
        self.stats["build_s"] += time.perf_counter() - t
        self.stats["builds"] += 1
        self.resident[key] = [handle, int(nbytes)]
        self.used += int(nbytes)
        if self.used > self.budget:  # the estimate was short: evict more now
            self._make_room(0)
        self.peak = max(self.peak, self.used)
        return handle

    def prepare(self, keys) -> None:
        """Make systems resident before a stream starts (first come first kept)."""
        for key in keys:
            self.ensure(key)

    # -- serving ------------------------------------------------------------
    @staticmethod
    def _produce(requests, inbox, t0, make_rhs):
        for req in sorted(requests, key=lambda r: r.arrival):
            rhs, err = None, None
            try:
                rhs = make_rhs(req)
            except Exception as e:  # reported with the request; the stream goes on
                err = f"request producer failed: {e!r}"
            delay = t0 + req.arrival - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            inbox.put((req, rhs, err))

    def run(self, requests, make_rhs: Callable[[Request], torch.Tensor] | None = None,
            keep: Callable[[Request], bool] | None = None) -> list[Result]:
        if make_rhs is None:
            make_rhs = lambda r: request_rhs(r, pin=torch.cuda.is_available())
        inbox: queue.Queue = queue.Queue()
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        prod = threading.Thread(target=self._produce, args=(requests, inbox, t0, make_rhs),
                                daemon=True)
        prod.start()
        pending: collections.deque = collections.deque()
        running: list = []
        free_slots = list(range(self.ex.slots))
        results: dict[int, Result] = {}
        expected = len(requests)

        def fail(req, msg):
            results[req.rid] = Result(req.rid, req.key, req.k, req.arrival, done=now(), error=msg)
            self.stats["failed"] += 1

        while len(results) < expected:
            progressed = False
            while True:  # arrivals
                try:
                    req, rhs, err = inbox.get_nowait()
                except queue.Empty:
                    break
                progressed = True
                if err is not None:
                    fail(req, err)
                else:
                    pending.append((req, rhs))
            for entry in list(running):  # completions
                slot, group, token = entry
                if self.ex.poll(token):
                    if len(group) == 1:
                        outs = [self.ex.finish(token)]
                    else:
                        outs = self.ex.finish_group(token)
                    t_done = now()
                    for (req, res), (x, its) in zip(group, outs):
                        res.done = t_done
                        res.iterations = its
                        res.x = x if keep is None or keep(req) else None
                        results[req.rid] = res
                    running.remove(entry)
                    free_slots.append(slot)
                    self.busy.discard(group[0][0].key)
                    progressed = True
            if free_slots and pending:  # dispatch, oldest first
                for item in list(pending):
                    if not free_slots:
                        break
                    req, rhs = item
                    if req.key in self.busy:
                        continue
                    try:
                        handle = self.ensure(req.key)
                    except Rejected as e:
                        pending.remove(item)
                        self.stats["rejected"] += 1
                        fail(req, str(e))
                        progressed = True
                        continue
                    if handle is None:
                        continue
                    group = [item]
                    merge = int(getattr(self.ex, "merge_rhs", 0) or 0)
                    if merge and req.k < merge:
                        # Later queued requests for the same system join this
                        # solve while the right-hand sides fit.
                        total = req.k
                        for other in pending:
                            if other is not item and other[0].key == req.key \
                                    and total + other[0].k <= merge:
                                group.append(other)
                                total += other[0].k
                    for g in group:
                        pending.remove(g)
                    slot = free_slots.pop()
                    t_start = now()
                    members = [(g[0], Result(g[0].rid, g[0].key, g[0].k, g[0].arrival,
                                             start=t_start)) for g in group]
                    try:
                        if len(group) == 1:
                            token = self.ex.start(slot, handle, req, rhs)
                        else:
                            token = self.ex.start_group(slot, handle, [g[0] for g in group],
                                                        [g[1] for g in group])
                    except (ValueError, RuntimeError) as e:
                        free_slots.append(slot)
                        for g in group:
                            fail(g[0], f"launch failed: {e}")
                        progressed = True
                        continue
                    self.busy.add(req.key)
                    running.append((slot, members, token))
                    progressed = True
            if (not prod.is_alive() and inbox.empty() and not pending and not running
                    and len(results) < expected):
                for req in requests:
                    if req.rid not in results:
                        fail(req, "request producer stopped before sending this request")
                break
            if not progressed:
                time.sleep(self.idle_sleep)
        prod.join(timeout=1.0)
        return [results[r.rid] for r in requests]


def summarize(results: list[Result]) -> dict:
    """Latency percentiles (ms), throughput and failure counts of a run."""
    ok = [r for r in results if r.ok]
    if not ok:
        return {"requests": len(results), "completed": 0, "failed": len(results)}
    lat = np.array([r.latency for r in ok]) * 1e3
    span = max(r.done for r in ok) - min(r.arrival for r in results)
    rhs = sum(r.k for r in ok)
    its = [i for r in ok for i in (r.iterations or [])]
    return {
        "requests": len(results),
        "completed": len(ok),
        "failed": len(results) - len(ok),
        "rhs_solved": rhs,
        "p50_ms": float(np.percentile(lat, 50)),
        "p90_ms": float(np.percentile(lat, 90)),
        "p99_ms": float(np.percentile(lat, 99)),
        "max_ms": float(lat.max()),
        "makespan_s": float(span),
        "solves_per_s": rhs / span if span > 0 else math.inf,
        "requests_per_s": len(ok) / span if span > 0 else math.inf,
        "iterations_mean": float(np.mean(its)) if its else 0.0,
        "iterations_max": int(max(its)) if its else 0,
    }
