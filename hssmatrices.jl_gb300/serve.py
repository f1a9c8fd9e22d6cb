"""Serving form: a request loop with resident factorizations and continuous batching.

Requests are either *factor* requests (a new HSS matrix: upload its generators,
factorize, keep the factorization resident) or *solve* requests (right-hand
sides against a resident factorization).

``HssServer`` keeps two CUDA streams busy at once.  The caller's thread admits
factor requests while the HBM budget allows (evicting least-recently-used
factorizations that no queued or running request needs) and launches each
admitted group as one batched factorization (``hss_batcher_factor``) on the
factor stream, without waiting for it.  A solve worker thread takes every solve
request whose matrix is resident (its factorization may still be running: the
solve stream waits for it on the device), joins the right-hand sides per matrix
and solves all of them in one launch sequence per tree level with
FP64-accurate refinement (``hss_batcher_solve``) on the solve stream.  Requests
that arrive while a batch runs are admitted by the next pass of either loop, so
factorizations of new matrices overlap solves against resident ones on the
device.  A request's result is the same alone and in any mix: every matrix of a
batch is an independent slot of the same kernels (the refinement of a batch
stops when all its columns meet the tolerance, so a column may get an extra
correction).

There is no CPU path: every step runs the CUDA library.
"""
from __future__ import annotations

import collections
import ctypes as C
import threading
import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _lib
from ._lib import check
from .linalg import DeviceHss, PREC, _stream


class Batcher:
    """Owner of an ``hss_batcher`` (merged task lists + buffers), one per stream."""

    def __init__(self):
        self.lib = _lib.load()
        self.handle = C.c_void_p()
        check(self.lib.hss_batcher_create(C.byref(self.handle)))

    def __del__(self):
        try:
            if self.handle:
                self.lib.hss_batcher_destroy(self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass

    def factor(self, devs, precision="fp32", stream=None):
        """Factorize several single-matrix plans in one launch sequence; returns factor handles."""
        k = len(devs)
        hs = (C.c_void_p * k)(*[d.handle for d in devs])
        out = (C.c_void_p * k)()
        check(self.lib.hss_batcher_factor(self.handle, k, hs, PREC[precision], out, _stream(stream)))
        return [ResidentFactor(self.lib, C.c_void_p(out[i]), PREC[precision]) for i in range(k)]

    def solve(self, factors, dBs, dXs, rows, rs, tol=1e-10, maxit=20, stream=None):
        """Solve factors[i] against dBs[i] (rows[i] x rs[i], column-major device buffers)."""
        k = len(factors)
        fs = (C.c_void_p * k)(*[f.handle for f in factors])
        B = (C.c_void_p * k)(*[_ptr(x) for x in dBs])
        X = (C.c_void_p * k)(*[_ptr(x) for x in dXs])
        ld = np.asarray(rows, dtype=np.int64)
        r = np.asarray(rs, dtype=np.int64)
        st = _lib.SolveStats()
        check(self.lib.hss_batcher_solve(self.handle, k, fs, B, _lib.iptr(ld), _lib.iptr(r), X, _lib.iptr(ld),
                                         float(tol), int(maxit), C.byref(st), _stream(stream)))
        return st


def _ptr(x):
    return x if isinstance(x, int) else x.data_ptr()


class ResidentFactor:
    def __init__(self, lib, handle, prec):
        self.lib = lib
        self.handle = handle
        self.prec = prec

    def nbytes(self):
        b = C.c_int64()
        check(self.lib.hss_factor_bytes(self.handle, C.byref(b)))
        return b.value

    def __del__(self):
        try:
            if self.handle:
                self.lib.hss_factor_destroy(self.handle)
                self.handle = C.c_void_p()
        except Exception:
            pass


@dataclass
class Request:
    rid: int
    kind: str                      # "factor" or "solve"
    arrival: float                 # seconds on the server's clock
    matrix: int                    # matrix id
    hss: object = None             # factor: the HssMatrix (host generators)
    rhs: object = None             # solve: torch tensor r x n (column-major n x r)
    done: Optional[float] = None
    out: object = None
    batch: int = -1
    nbytes: int = 0
    ready: object = None           # solve: event after which rhs is valid (recorded at submit)


@dataclass
class Resident:
    dev: DeviceHss
    factor: ResidentFactor
    nbytes: int
    n: int
    last_use: float = 0.0
    ready: object = None           # event recorded after the factorization on the factor stream


class HssServer:
    """Continuous-batching HSS factor/solve server on one GPU (two streams, a solve worker).

    ``overlap=False`` runs the same batches one after the other on the caller's
    thread (factor batch, then solve batch, each waited for): the form without
    overlap, kept for comparison."""

    def __init__(self, budget_bytes=150 * 10**9, precision="fp32", tol=1e-10, maxit=20,
                 max_factor_batch=32, overlap=True):
        import torch
        self.torch = torch
        self.budget = int(budget_bytes)
        self.precision = precision
        self.tol = tol
        self.maxit = maxit
        self.max_factor_batch = max_factor_batch
        self.overlap = overlap
        self.fstream = torch.cuda.Stream()
        self.sstream = torch.cuda.Stream()
        self.fbatcher = Batcher()
        self.sbatcher = Batcher()
        self.cv = threading.Condition()
        self.resident: "collections.OrderedDict[int, Resident]" = collections.OrderedDict()
        self.pending_factor: "collections.deque[Request]" = collections.deque()
        self.pending_solve: "list[Request]" = []
        self.inflight = collections.deque()    # (event, factor requests) on the factor stream
        self.busy = set()                      # matrices of the running solve batch
        self.completed = []
        self.used = 0
        self.batches = 0
        self.factor_batches = 0
        self.solve_batches = 0
        self.evictions = 0
        self.reloads = 0
        self.overlapped = 0            # factor batches launched while a solve batch ran
        self.matrices = {}             # matrix id -> host HssMatrix (re-admission after eviction)
        self.now_fn = time.perf_counter
        self.error = None
        self._stop = False
        self._worker = None

    # -- accounting --------------------------------------------------------
    @staticmethod
    def estimate_bytes(hss, precision):
        """Generators (+ their FP32-pair copy) + factor storage + workspaces, from the sizes."""
        from .packing import pack_cached
        _table, packed = pack_cached(hss)
        gen = packed.size * 8
        m = hss.size()[0]
        fac_elems = 2 * packed.size + 8 * m     # factor blocks, reflector copies, tau vectors
        item = 4 if precision == "fp32" else 8
        # FP32 + refinement: the generators' pair copy, and the bf16 slices of the
        # leaf blocks for the tensor-core residual (7 x 2 bytes per entry)
        extra = 3 * gen if precision == "fp32" else 0
        return gen + extra + fac_elems * item + 64 * m * 8

    def _account(self, res):
        """Replaces a resident matrix's share of the budget by the device memory its
        handle and factorization hold now (lock held)."""
        b = C.c_int64()
        check(res.dev.lib.hss_device_bytes(res.dev.handle, res.factor.handle, C.byref(b)))
        self.used += b.value - res.nbytes
        res.nbytes = b.value

    def _evict_for(self, need, keep):
        while self.used + need > self.budget:
            victim = None
            for mid, res in self.resident.items():    # least recently used first
                if mid not in keep:
                    victim = mid
                    break
            if victim is None:
                return False
            res = self.resident.pop(victim)
            self.used -= res.nbytes
            self.evictions += 1
        return True

    # -- request intake ------------------------------------------------------
    def submit(self, req: Request):
        if req.kind == "solve" and req.rhs is not None:
            req.ready = self.torch.cuda.Event()
            req.ready.record()   # the caller's stream: rhs is valid after this point
        with self.cv:
            if req.kind == "factor":
                self.matrices[req.matrix] = req.hss
                self.pending_factor.append(req)
            else:
                self.pending_solve.append(req)
            self.cv.notify_all()

    # -- factor side (the caller's thread) -------------------------------------
    def _admit_and_factor(self):
        """Admit queued factor requests within the budget and launch them as one
        batch on the factor stream; does not wait for the device."""
        with self.cv:
            keep = {r.matrix for r in self.pending_solve} | self.busy
            for _ev, reqs in self.inflight:
                keep |= {r.matrix for r in reqs}
            # a matrix evicted while solves for it were still to come is loaded again
            queued = {r.matrix for r in self.pending_factor}
            for mid in {r.matrix for r in self.pending_solve}:
                if mid not in self.resident and mid not in queued and mid in self.matrices:
                    self.pending_factor.appendleft(Request(-1, "factor", self.now_fn(), mid,
                                                           hss=self.matrices[mid]))
                    queued.add(mid)
                    self.reloads += 1
            admitted = []
            while self.pending_factor and len(admitted) < self.max_factor_batch:
                req = self.pending_factor[0]
                need = self.estimate_bytes(req.hss, self.precision)
                if need > self.budget:
                    raise MemoryError(f"matrix {req.matrix} needs {need} bytes, above the budget {self.budget}")
                if not self._evict_for(need, keep | {r.matrix for r in admitted}):
                    break
                self.pending_factor.popleft()
                self.used += need
                req.nbytes = need
                admitted.append(req)
        if not admitted:
            return False
        devs = [DeviceHss(r.hss) for r in admitted]
        with self.cv:
            if self.busy:
                self.overlapped += 1   # launched while a solve batch is on the device
        factors = self.fbatcher.factor(devs, self.precision, stream=self.fstream)
        ev = self.torch.cuda.Event()
        ev.record(self.fstream)
        with self.cv:
            for r, d, f in zip(admitted, devs, factors):
                res = Resident(d, f, r.nbytes, d.n, self.now_fn(), ev)
                self._account(res)
                self.resident[r.matrix] = res
                self.resident.move_to_end(r.matrix)
            self.inflight.append((ev, admitted))
            self.factor_batches += 1
            self.batches += 1
            self.cv.notify_all()
        return True

    def _reap_factors(self, wait=False):
        """Completes the factor requests of finished factor batches."""
        with self.cv:
            while self.inflight:
                ev, reqs = self.inflight[0]
                if wait:
                    ev.synchronize()
                elif not ev.query():
                    break
                self.inflight.popleft()
                t = self.now_fn()
                for r in reqs:
                    if r.rid < 0:
                        continue   # internal re-admission
                    r.done = t
                    r.batch = self.factor_batches
                    self.completed.append(r)

    # -- solve side (the worker thread, or the caller's without overlap) ---------
    def _take_solves(self):
        """Every queued solve whose matrix is resident, grouped per matrix (lock held)."""
        ready = [r for r in self.pending_solve if r.matrix in self.resident]
        if not ready:
            return None
        self.pending_solve = [r for r in self.pending_solve if r.matrix not in self.resident]
        groups = collections.OrderedDict()
        for r in ready:
            groups.setdefault(r.matrix, []).append(r)
        batch = []
        for mid, reqs in groups.items():
            res = self.resident[mid]
            res.last_use = self.now_fn()
            self.resident.move_to_end(mid)
            batch.append((mid, res, reqs))
        self.busy = set(groups)
        return batch

    def _run_solves(self, batch):
        torch = self.torch
        st = self.sstream
        facs, dBs, dXs, rows, rs = [], [], [], [], []
        for _mid, res, reqs in batch:
            st.wait_event(res.ready)             # the factorization, on the device
            for q in reqs:
                if q.ready is not None:
                    st.wait_event(q.ready)       # the right-hand sides
        with torch.cuda.stream(st):
            for _mid, res, reqs in batch:
                B = torch.cat([q.rhs for q in reqs], dim=0) if len(reqs) > 1 else reqs[0].rhs
                facs.append(res.factor)
                dBs.append(B)
                dXs.append(torch.empty_like(B))
                rows.append(res.n)
                rs.append(B.shape[0])
        self.sbatcher.solve(facs, dBs, dXs, rows, rs, tol=self.tol, maxit=self.maxit, stream=st)
        st.synchronize()
        t = self.now_fn()
        with self.cv:
            self.solve_batches += 1
            self.batches += 1
            for _mid, res, _reqs in batch:
                self._account(res)          # workspaces grown by the solve
            for (_mid, _res, reqs), X in zip(batch, dXs):
                c0 = 0
                for q in reqs:
                    q.out = X[c0:c0 + q.rhs.shape[0]]
                    c0 += q.rhs.shape[0]
                    q.done = t
                    q.batch = self.solve_batches
                    self.completed.append(q)
            self.busy = set()
            self.cv.notify_all()

    def _solve_loop(self):
        try:
            while True:
                with self.cv:
                    batch = None
                    while not self._stop:
                        batch = self._take_solves()
                        if batch is not None:
                            break
                        self.cv.wait(0.01)
                    if batch is None:
                        return
                self._run_solves(batch)
        except BaseException as e:   # surfaced on the caller's thread by pump()
            with self.cv:
                self.error = e
                self.busy = set()
                self.cv.notify_all()

    # -- driving -----------------------------------------------------------------
    def start(self, now_fn=None):
        if now_fn is not None:
            self.now_fn = now_fn
        if self.overlap and self._worker is None:
            self._stop = False
            self._worker = threading.Thread(target=self._solve_loop, name="hss-solve", daemon=True)
            self._worker.start()

    def stop(self):
        if self._worker is not None:
            with self.cv:
                self._stop = True
                self.cv.notify_all()
            self._worker.join()
            self._worker = None
        self._reap_factors(wait=True)

    def pump(self):
        """One pass of the caller's loop: launch admitted factorizations, complete
        finished ones (and, without overlap, run the solve batch); returns the
        requests completed since the last call."""
        if self.error is not None:
            raise self.error
        launched = self._admit_and_factor()
        if not self.overlap:
            if launched:
                self._reap_factors(wait=True)
            with self.cv:
                batch = self._take_solves()
            if batch is not None:
                self._run_solves(batch)
        self._reap_factors()
        with self.cv:
            done, self.completed = self.completed, []
        return done

    def step(self, now_fn):
        """Runs the queued work to completion without overlap (one factor batch,
        then one solve batch); returns the completed requests."""
        self.now_fn = now_fn
        overlap, self.overlap = self.overlap, False
        try:
            return self.pump()
        finally:
            self.overlap = overlap

    def idle(self):
        with self.cv:
            return (not self.pending_factor and not self.pending_solve and not self.inflight
                    and not self.busy and not self.completed)


def run_stream(server, requests, time_scale=1.0, poll=0.0):
    """Replay requests (sorted by arrival, seconds) in real time against ``server``;
    returns the completed requests with arrival/done on one clock."""
    t0 = time.perf_counter()

    def now():
        return (time.perf_counter() - t0) / time_scale

    server.start(now)
    i = 0
    out = []
    n = len(requests)
    try:
        while len(out) < n:
            t = now()
            while i < n and requests[i].arrival <= t:
                server.submit(requests[i])
                i += 1
            out.extend(server.pump())
            if len(out) >= n:
                break
            if server.idle() and i < n:
                wait = (requests[i].arrival - now()) * time_scale
                if wait > 0:
                    time.sleep(min(wait, 0.001))
            elif poll:
                time.sleep(poll)
            else:
                time.sleep(0.0002)   # leave the interpreter to the solve worker
    finally:
        server.stop()
    out.extend(server.pump())
    return out


def synthetic_requests(n_requests=10000, seed=3, rate=2000.0, factor_frac=0.2, n_range=(2048, 65536),
                       k_range=(16, 48), leafsize=128, r_range=(1, 32), pool_size=32, recent=16,
                       device="cuda"):
    """The serving workload: Poisson arrivals at `rate` per second; `factor_frac` are
    factor requests for a new matrix (n log-uniform in n_range, rank uniform in
    k_range, `leafsize`), the rest solve requests with r uniform in r_range against
    one of the `recent` most recently factored matrices.  Matrices come from a
    seeded pool of `pool_size` synthetic trees (each factor request gets a new
    matrix id and uploads its pool entry); right-hand sides are N(0,1) on the device.
    The first request is a factor request.  Each pool matrix is packed into the
    upload layout here, when the request is made (a client sends a matrix in
    that layout), not inside the serving loop."""
    import torch
    from .packing import pack_cached
    from .synthetic import synthetic_hss
    rng = np.random.default_rng(seed)
    pool = []
    for _ in range(pool_size):
        n = int(round(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1])))))
        k = int(rng.integers(k_range[0], k_range[1] + 1))
        pool.append(synthetic_hss(n, leafsize, k, rng))
        pack_cached(pool[-1])
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    t = 0.0
    reqs = []
    factored = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        if i == 0 or rng.random() < factor_frac:
            mid = len(factored)
            h = pool[mid % pool_size]
            factored.append((mid, h.size()[0]))
            reqs.append(Request(i, "factor", t, mid, hss=h))
        else:
            mid, n = factored[-1 - int(rng.integers(0, min(recent, len(factored))))]
            r = int(rng.integers(r_range[0], r_range[1] + 1))
            rhs = torch.randn((r, n), dtype=torch.float64, device=device, generator=gen)
            reqs.append(Request(i, "solve", t, mid, rhs=rhs))
    return reqs, pool
