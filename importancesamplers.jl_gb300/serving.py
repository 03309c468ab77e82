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
from .results import RoundError, SamplerExecutionError
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


def serve_latency_summary(results):
    """p50 / p99 latency (seconds) and retained weighted samples per second."""
    lat = np.array([r.latency for r in results])
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "requests": len(results)}
