"""Continuous serving of independent AMIS posterior runs.

Requests (one posterior each: a target, an initial proposal, a round schedule
and a seed) arrive over time. The loop admits a request as soon as it has
arrived, a stream slot is free and its device footprint fits the memory
budget. Each admitted run gets its own CUDA stream and its own scratch
buffers (a workspace scope). All of its kernels (draws, target, retrospective
denominators, weights, summaries, moments, FP64 fits) are queued on that stream
without a host synchronisation, by one native call (issm_amis_run) for
Gaussian factor proposals with a native target, so the device overlaps runs of
different dimension and budget and the host's cost per run stays small. The loop polls the runs' completion events, reads back
each finished run's summaries and posterior mean, frees its buffers and
admits the next. A run's results depend only on its own inputs and seed: the
same run alone or in the mix gives bitwise the same numbers.

Not done here: merging the kernels of many small runs into one launch (every
run issues its own launches, from native code).
"""
import heapq
import itertools
import time

import numpy as np
import torch

from . import native
from .methods import AMIS
from .results import AMISRoundError, RoundError, SamplerExecutionError
from .sampler import (SamplerBusyError, _finish_moment_summary, _moment_body, _native_body, native_body_eligible,
                      prepare_sampler)


class ServeRequest:
    """One posterior run: AMIS(proposal; rounds, round_size) on `target`."""

    def __init__(self, rid, target, proposal, rounds, round_size, seed, arrival=0.0):
        self.rid, self.target, self.proposal = rid, target, proposal
        self.rounds, self.round_size, self.seed, self.arrival = int(rounds), int(round_size), int(seed), float(arrival)

    @property
    def samples(self):
        return self.rounds * self.round_size

    def footprint(self):
        """Device bytes the run holds: retained samples and their four
        per-sample arrays, the proposal history and its inverse factors, and
        scratch (an upper estimate)."""
        d = self.proposal.dimension
        es = np.dtype(self.proposal.dtype).itemsize
        n = self.samples
        dp = 16 if d <= 16 else 32 if d <= 32 else 64
        history = self.rounds * (d * d + d + 1) * es + self.rounds * dp * dp * 4
        scratch = (self.rounds + 4) * dp * (4 * dp + 64) * 2 + (1 << 22)
        return n * d * es + n * (3 * es + 8) + history + scratch


class ServeResult:
    """A finished run: posterior mean, final-round log Z and ESS, timings; or,
    when the run failed (AMISRoundError and the like), `error` with NaN
    outputs. A failed run never stops the loop."""

    def __init__(self, request, posterior_mean, logz, ess, start, end, error=None):
        self.rid = request.rid
        self.posterior_mean, self.logz, self.ess = posterior_mean, logz, ess
        self.arrival, self.start, self.end = request.arrival, start, end
        self.error = error

    @property
    def latency(self):
        return self.end - self.arrival


class _Running:
    def __init__(self, request, sampler, stream, event, start):
        self.request, self.sampler, self.stream, self.event, self.start = request, sampler, stream, event, start


class ServeLoop:
    """Admit, launch and retire AMIS runs on one GPU (see the module docstring)."""

    def __init__(self, device="cuda", memory_budget=8 << 30, max_inflight=8, precision=native.PREC_BF16):
        native.require()
        self.device = torch.device(device)
        self.memory_budget = int(memory_budget)
        self.max_inflight = int(max_inflight)
        self.precision = precision
        self.streams = [torch.cuda.Stream(self.device) for _ in range(self.max_inflight)]
        self._ids = itertools.count()

    def _form(self, request):
        # tensor-core forms need FP32 factor proposals with d <= 64
        p = request.proposal
        if p.dtype == np.float32 and p.dimension <= 64:
            return self.precision
        return native.PREC_NATIVE

    def _launch(self, request, stream, now):
        """Prepare and issue one run on `stream`. Returns the running run, or
        the exception that stopped it from being issued (an allocation
        failure, an argument the library rejects): that run is reported
        failed and its scratch released, and the loop goes on."""
        scope = ("serve", next(self._ids))
        try:
            with torch.cuda.stream(stream), native.workspace_scope(scope):
                s = prepare_sampler(request.seed, request.target,
                                    AMIS(request.proposal, rounds=request.rounds, round_size=request.round_size),
                                    device=self.device, precision=self._form(request), graphs=False)
                if s.busy:
                    raise SamplerBusyError("prepared sampler is already running")
                s.busy = True
                if native_body_eligible(s):
                    _native_body(s)  # every launch of the run in one native call
                else:
                    _moment_body(s, False)
                event = torch.cuda.Event()
                event.record(stream)
        except Exception as e:  # noqa: BLE001 - any launch failure fails this run only
            # work issued before the failure may still be running on the
            # stream: let it finish before the scope's buffers are freed
            stream.synchronize()
            native.release_scope(scope)
            return e
        s.scope = scope
        return _Running(request, s, stream, event, now)

    def _retire(self, run, now):
        s = run.sampler
        error = None
        try:
            with torch.cuda.stream(run.stream), native.workspace_scope(s.scope):
                try:
                    pm, logz, ess = _finish_moment_summary(s)
                except (RoundError, SamplerExecutionError, RuntimeError) as e:  # this run failed; the others go on
                    d = run.request.proposal.dimension
                    pm, logz, ess, error = np.full(d, np.nan), float("nan"), 0.0, e
                finally:
                    s.busy = False
        finally:
            native.release_scope(s.scope)
        return ServeResult(run.request, pm, logz, ess, run.start, now, error)

    def run(self, requests, clock=time.perf_counter):
        """Serve `requests` (their `arrival` is seconds after the call) and
        return their results in completion order."""
        pending = sorted(requests, key=lambda r: r.arrival)
        for r in pending:
            if r.footprint() > self.memory_budget:
                raise ValueError(f"request {r.rid} needs {r.footprint()} bytes, more than the budget")
        t0 = clock()
        free = list(range(self.max_inflight))
        running, results, used = {}, [], 0
        queue = []  # arrived, waiting for a slot or memory (FIFO by arrival)
        i = 0
        while i < len(pending) or queue or running:
            now = clock() - t0
            while i < len(pending) and pending[i].arrival <= now:
                heapq.heappush(queue, (pending[i].arrival, i, pending[i]))
                i += 1
            # retire completed runs
            for slot, run in list(running.items()):
                if run.event.query():
                    results.append(self._retire(run, clock() - t0))
                    used -= run.request.footprint()
                    del running[slot]
                    free.append(slot)
            # admit in arrival order while a slot and the memory budget allow
            while queue and free and used + queue[0][2].footprint() <= self.memory_budget:
                _, _, req = heapq.heappop(queue)
                slot = free.pop()
                launched = self._launch(req, self.streams[slot], clock() - t0)
                if isinstance(launched, _Running):
                    running[slot] = launched
                    used += req.footprint()
                else:  # not issued: reported failed now, slot and memory stay free
                    t = clock() - t0
                    results.append(ServeResult(req, np.full(req.proposal.dimension, np.nan), float("nan"), 0.0, t, t,
                                               launched))
                    free.append(slot)
            if not running and not queue and i < len(pending):
                time.sleep(max(0.0, min(pending[i].arrival - (clock() - t0), 0.001)))
            elif running:
                time.sleep(0.0002)
        return results


GROUP_TILE, GROUP_MOMENT_SAMPLES, GROUP_MOMENT_WORDS = 128, 2048, 2145
_RUN_FIELDS = ["d", "rounds", "round", "n_round", "n_old", "seed", "normal_offset", "blk_new0", "blk_all0",
               "blk_mom0", "nmom", "samples", "logtargets", "lognum", "logweights", "loc", "fac", "lognorm",
               "cand_loc", "cand_fac", "cand_lognorm", "t_mode", "t_chol", "summaries", "mean", "cov", "failures",
               "partial", "mpartial", "t_const", "logcount"]
_COL = {name: k for k, name in enumerate(_RUN_FIELDS)}


def _cdiv(a, b):
    return -(-a // b)


class _Prep:
    """Host side of one grouped run, computed off the serving thread: the
    target's exact mode-centred form from its sufficient statistics, the byte
    layout of the run's single device allocation, and the bytes admission
    writes (zeroed failure words, the target's mode and factor, the history's
    slot 0)."""

    # 256-byte aligned slices of one allocation; the head (up to the end of
    # slot 0 of the factors) is written by one host-to-device copy
    _HEAD = (("failures", 8), ("t_mode", 4), ("t_chol", 4), ("lognorm", 4), ("loc", 4), ("fac", 4))
    _REST = (("cand_loc", 4), ("cand_fac", 4), ("cand_lognorm", 4), ("samples", 4), ("logtargets", 4),
             ("lognum", 4), ("logweights", 4), ("summaries", 8), ("mean", 8), ("cov", 8), ("partial", 8),
             ("mpartial", 8))

    def __init__(self, request):
        p, tgt = request.proposal, request.target
        d, R, n = p.dimension, request.rounds, request.round_size
        self.request, self.d, self.R, self.n = request, d, R, n
        X, y, s2, pv = tgt.X, tgt.y, tgt.sigma ** 2, tgt.prior_var
        A = X.T @ X / s2 + np.eye(d) / pv
        mode = np.linalg.solve(A, X.T @ y / s2)
        r = y - X @ mode
        self.t_const = float(-0.5 * len(y) * np.log(2 * np.pi * s2) - 0.5 * float(r @ r) / s2
                             - 0.5 * d * np.log(2 * np.pi * pv) - 0.5 * float(mode @ mode) / pv)
        U = np.linalg.cholesky(A).T  # A = U^T U, U upper
        count = {"failures": 3 * R, "t_mode": d, "t_chol": d * d, "lognorm": R, "loc": R * d, "fac": R * d * d,
                 "cand_loc": d, "cand_fac": d * d, "cand_lognorm": 1, "samples": R * n * d, "logtargets": R * n,
                 "lognum": R * n, "logweights": R * n, "summaries": 3 * R, "mean": d, "cov": d * d,
                 "partial": 3 * _cdiv(R * n, GROUP_TILE),
                 "mpartial": GROUP_MOMENT_WORDS * _cdiv(R * n, GROUP_MOMENT_SAMPLES)}
        self.off, o = {}, 0
        for name, es in self._HEAD + self._REST:
            self.off[name] = o
            o += _cdiv(count[name] * es, 256) * 256
        self.nbytes = o
        head = np.zeros(self.off["fac"] + 4 * d * d, dtype=np.uint8)
        f32 = head.view(np.float32)

        def put(name, values):
            a = self.off[name] // 4
            f32[a:a + values.size] = values

        put("t_mode", mode.astype(np.float32))
        put("t_chol", np.ascontiguousarray(U.T, dtype=np.float32).reshape(-1))  # U column-major
        put("lognorm", np.array([p.lognormalizer], dtype=np.float32))
        put("loc", np.asarray(p.location, dtype=np.float32))
        put("fac", np.ascontiguousarray(p.factor_matrix().T, dtype=np.float32).reshape(-1))  # L column-major
        self.head = head


class _GroupedRun:
    """The device state of one admitted run: one allocation carved into the
    issm_group_run arrays, its head written by one asynchronous copy from
    pinned memory, and the run's fixed descriptor fields as one table row."""

    def __init__(self, prep, device, start):
        self.prep, self.request, self.start, self.round = prep, prep.request, start, 0
        self.d, self.R, self.n = prep.d, prep.R, prep.n
        self.buf = torch.empty(prep.nbytes, dtype=torch.uint8, device=device)
        # pinned (cached host allocator) and asynchronous: admission never waits for the device
        self.buf[:prep.head.size].copy_(torch.from_numpy(prep.head).pin_memory(), non_blocking=True)
        base = self.buf.data_ptr()
        row = np.zeros(len(_RUN_FIELDS), dtype=np.int64)
        row[_COL["d"]], row[_COL["rounds"]], row[_COL["n_round"]] = self.d, self.R, self.n
        row[_COL["seed"]] = np.uint64(self.request.seed & (2 ** 64 - 1)).view(np.int64)
        for name, o in prep.off.items():
            row[_COL[name]] = base + o
        row.view(np.float64)[_COL["t_const"]] = prep.t_const
        row.view(np.float64)[_COL["logcount"]] = float(np.float32(np.log(self.n)))
        self.row = row

    def nbytes(self):
        return self.prep.nbytes

    def result_views(self):
        """The bytes read back when the run finishes: failure words, the last
        round's summary, the posterior mean."""
        o = self.prep.off
        s = o["summaries"] + 24 * (self.R - 1)
        return [self.buf[o["failures"]:o["failures"] + 24 * self.R], self.buf[s:s + 24],
                self.buf[o["mean"]:o["mean"] + 8 * self.d]]


class GroupedServeLoop:
    """Continuous batching of AMIS linear-regression posterior runs (Gaussian
    factor proposals, FP32, d <= 64) with one launch per phase per step for
    every in-flight run (issm_group_step).

    Each step advances every in-flight run by one round: the host writes one
    descriptor row per run (its arrays, round, random-stream position and
    block offsets), copies the table to the device and issues seven kernels;
    runs of any dimension, budget and round share the launches. A request
    joins at the next step once it has arrived and the memory budget allows
    (its host preparation, the target's sufficient statistics, mode and
    factor, runs on the serving thread: BLAS calls from several threads at
    once oversubscribe the host's cores). A run that finished its last round
    is read back asynchronously (failure words, final summary and posterior
    mean, one copy for every run that finished at that step) and its memory
    returned. At most `lookahead` steps are in flight, so admissions follow
    the device. A run's numbers depend only on its own inputs and seed: alone
    and in any mix they are bitwise the same."""

    def __init__(self, device="cuda", memory_budget=16 << 30, max_inflight=4096, lookahead=2):
        native.require()
        self.device = torch.device(device)
        self.memory_budget = int(memory_budget)
        self.max_inflight = int(max_inflight)
        self.lookahead = int(lookahead)
        self.stream = torch.cuda.current_stream(self.device)

    @staticmethod
    def eligible(request):
        from .proposals import FACTOR, GAUSSIAN
        from .targets import LinearRegressionTarget

        p = request.proposal
        return (isinstance(request.target, LinearRegressionTarget) and p.family == GAUSSIAN and
                p.scale_kind == FACTOR and p.dtype == np.float32 and p.dimension <= 64)

    @staticmethod
    def _table(runs):
        """The step's descriptor table: the runs' fixed rows and, per run,
        its round, retained count, normal-stream position and block offsets
        (exclusive prefix sums of its block counts)."""
        t = np.stack([g.row for g in runs])
        rnd = np.array([g.round for g in runs], dtype=np.int64)
        n = t[:, _COL["n_round"]]
        d = t[:, _COL["d"]]
        nall = (rnd + 1) * n
        bn = -(-n // GROUP_TILE)
        ba = -(-nall // GROUP_TILE)
        bm = -(-nall // GROUP_MOMENT_SAMPLES)
        t[:, _COL["round"]] = rnd
        t[:, _COL["n_old"]] = rnd * n
        # each round takes n d + 8 elements of the run's normal stream
        t[:, _COL["normal_offset"]] = rnd * (n * d + 8)
        for col, cnt in (("blk_new0", bn), ("blk_all0", ba), ("blk_mom0", bm)):
            t[:, _COL[col]] = np.cumsum(cnt) - cnt
        t[:, _COL["nmom"]] = bm
        return t, int(bn.sum()), int(ba.sum()), int(bm.sum())

    def run(self, requests, clock=time.perf_counter):
        pending = sorted(requests, key=lambda r: r.arrival)
        for r in pending:
            if not self.eligible(r):
                raise ValueError(f"request {r.rid}: the grouped loop serves linear-regression targets with FP32 "
                                 "Gaussian factor proposals of d <= 64")
        native.lib()
        t0 = clock()
        queue, active, reading, results = [], [], [], []
        preps = {}  # request id -> _Prep of the queue head held back by the memory budget
        steps = []  # (event, host table, device table) of steps in flight
        used, i = 0, 0
        while i < len(pending) or queue or active or reading:
            now = clock() - t0
            while i < len(pending) and pending[i].arrival <= now:
                queue.append(pending[i])
                i += 1
            # decode the read-backs that have landed
            if reading:
                landed = [x for x in reading if x[2].query()]
                if landed:
                    reading = [x for x in reading if all(x is not y for y in landed)]
                    for runs, host, _ in landed:
                        results.extend(self._decode(runs, host.numpy(), clock() - t0))
                        used -= sum(g.nbytes() for g in runs)
            # admit in arrival order while the in-flight cap and the memory budget allow
            while queue and len(active) < self.max_inflight:
                request = queue[0]
                if request.rid not in preps:
                    try:
                        preps[request.rid] = _Prep(request)
                    except Exception as e:  # a target the preparation rejects fails alone
                        queue.pop(0)
                        results.append(ServeResult(request, np.full(request.proposal.dimension, np.nan),
                                                   float("nan"), 0.0, clock() - t0, clock() - t0, e))
                        continue
                prep = preps[request.rid]
                if used + prep.nbytes > self.memory_budget and (active or reading):
                    break
                queue.pop(0)
                del preps[request.rid]
                active.append(_GroupedRun(prep, self.device, clock() - t0))
                used += prep.nbytes
            if active:
                # at most `lookahead` steps in flight
                while len(steps) >= self.lookahead:
                    steps.pop(0)[0].synchronize()
                table, bn, ba, bm = self._table(active)
                host = torch.from_numpy(table).pin_memory()
                dev = torch.empty_like(host, device=self.device)
                dev.copy_(host, non_blocking=True)
                native.call("issm_group_step", dev.data_ptr(), len(active), bn, ba, bm, self.stream.cuda_stream)
                ev = torch.cuda.Event()
                ev.record(self.stream)
                steps.append((ev, host, dev))
                still, done = [], []
                for g in active:
                    g.round += 1
                    (done if g.round == g.R else still).append(g)
                active = still
                if done:
                    reading.append(self._read_back(done))
            elif not queue and i < len(pending):
                time.sleep(max(0.0, min(pending[i].arrival - (clock() - t0), 0.001)))
            elif reading:
                time.sleep(0.0002)
        return results

    def _read_back(self, runs):
        """Stream-ordered after the runs' last step: one gather and one
        asynchronous copy into pinned memory for every run that finished."""
        packed = torch.cat([v for g in runs for v in g.result_views()])
        host = torch.empty(packed.numel(), dtype=torch.uint8, pin_memory=True)
        host.copy_(packed, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(self.stream)
        return runs, host, ev

    def _decode(self, runs, packed, now):
        out, o = [], 0
        for g in runs:
            words = packed[o:o + 24 * g.R].view(np.int64).reshape(g.R, 3)
            o += 24 * g.R
            m, s, s2 = packed[o:o + 24].view(np.float64)
            o += 24
            mean = packed[o:o + 8 * g.d].view(np.float64).copy()
            o += 8 * g.d
            error = None
            for t in range(g.R):
                if words[t][0] != 0:
                    from .sampler import _raise_failures

                    try:
                        _raise_failures(words[t], AMISRoundError, t + 1)
                    except AMISRoundError as e:
                        error = e
                    break
            total = g.R * g.n
            logz = float(m + np.log(s) - np.log(total)) if s > 0 else float("-inf")
            ess = float(s * s / s2) if s > 0 else 0.0
            if error is not None:
                mean, logz, ess = np.full(g.d, np.nan), float("nan"), 0.0
            out.append(ServeResult(g.request, mean, logz, ess, g.start, now, error))
        return out


def serve_latency_summary(results):
    """p50 / p99 latency (seconds) and retained weighted samples per second."""
    lat = np.array([r.latency for r in results])
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "requests": len(results)}
