"""Headline benchmark: AMIS weighted samples/s on the d = 64 Student-t
workload (40 rounds x 50,000 samples, 2,000,000 retained weighted samples),
through the public sampler API, with the log-Z and posterior-mean error
reported beside the rate.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision bf16|tf32|fp32] [--impl gb300|reference]

The headline line is the BF16 x3 tensor-core form (Mahalanobis contraction and
moments on tcgen05, FP64 Cholesky and log-Z sums); "forms" reports the TF32
and plain FP32 forms on the same GPU and workload beside it, timed from the
same random-stream position.

One step = one complete AMIS run (draw, target, retrospective
balance-heuristic denominators, weights, summaries, weighted moments and FP64
Cholesky fits for all 40 rounds) on device-resident problem data. `e2e`
repeats the step through the same public API starting from host arrays
(target and initial proposal copied in) and reading the run's summaries and
posterior mean back. Under torchrun every rank runs an independent replica
(the path has no cross-sample exchange), timed between barriers, max over ranks.

Accuracy: every timed step's |log Zhat - log Z| and posterior-mean error
against the analytic target; the arithmetic of each form against FP64 with
the adaptation held fixed (the FP64 run's samples re-weighed under its own
proposal history); and the adaptive runs from the same normals (device FP64
and the FP64 oracle on the host cores, whose run time is the CPU baseline).

`--impl reference` times the CPU restatement of the reference's threaded AMIS
(FP64, all host cores) on the full workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

D, ROUNDS, ROUND_SIZE, DOF = 64, 40, 50_000, 5.0
WORKLOAD = "AMIS d=64, Student-t target (nu=5), 40 rounds x 50,000 samples, factor-Gaussian proposals"
METRIC = "AMIS weighted samples/s at fixed logZ error"


def problem(seed=20261203):
    """Seeded synthetic C4 inputs: scale factor L (N(0, 0.3^2) below the
    diagonal, 1 + |N(0,1)| on it), location 0, initial proposal N(0, 9 I)."""
    rng = np.random.default_rng(seed)
    L = np.tril(rng.normal(scale=0.3, size=(D, D)), -1) + np.diag(1.0 + np.abs(rng.normal(size=D)))
    return np.zeros(D), L, np.zeros(D), 3.0 * np.eye(D)


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu_index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


FP32_RIDGE = float(np.sqrt(np.finfo(np.float32).eps))
# BASELINE's accuracy gate: |log Zhat - log Z| and the posterior-mean error
GATE = {"abs_logz_error": 1e-3, "posterior_mean_max_abs_error": 1e-2}


def oracle_amis(normals, round_size=ROUND_SIZE, rounds=ROUNDS, regularization=None):
    """One oracle AMIS run (FP64, OpenMP on every host core) on fed normals;
    returns (seconds, threads, result dict)."""
    from oracle import oracle as orc

    loc, L, p_loc, p_fac = problem()
    tgt = orc.TargetView(orc.TARGET_STUDENT_T, D, a=loc, b=L, p0=DOF)
    t0 = time.perf_counter()
    out = orc.amis_run(tgt, D, p_loc, p_fac, [round_size] * rounds, normals, regularization=regularization)
    return time.perf_counter() - t0, orc.num_threads(), out


def oracle_posterior_mean(out):
    lw = out["logweights"]
    w = np.exp(lw - lw.max())
    return (w / w.sum()) @ out["samples"].reshape(-1, D)


def run_reference(args):
    """The reference's CPU path (the FP64 OpenMP restatement of its threaded
    AMIS) on the full workload, 40 rounds x 50,000 samples, every step."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle import oracle as orc

    orc.build()
    normals = orc.philox_normals(11, 0, ROUND_SIZE * ROUNDS * D)
    for _ in range(args.warmup):
        oracle_amis(normals)
    times, errs, merrs = [], [], []
    for _ in range(args.steps):
        dt, cores, out = oracle_amis(normals)
        times.append(dt)
        errs.append(abs(float(out["round_logz"][-1])))
        merrs.append(float(np.max(np.abs(oracle_posterior_mean(out)))))
    total = ROUND_SIZE * ROUNDS
    value = total * len(times) / sum(times)
    sample = f"the full workload: 40 rounds x {ROUND_SIZE} samples (d=64), FP64, one complete AMIS run per step"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "weighted samples/s",
            "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded C4 inputs)",
            "config": {"workload": WORKLOAD, "d": D, "rounds": ROUNDS, "round_size": ROUND_SIZE, "sample": sample,
                       "backend": "CPU oracle restatement of the reference's threaded AMIS (OpenMP)"},
            "cpu_baseline": {"value": value, "unit": "weighted samples/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "weighted samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "accuracy": {"abs_logz_error": errs[-1], "posterior_mean_max_abs_error": merrs[-1],
                         "gate": GATE, "passes_gate": bool(errs[-1] <= GATE["abs_logz_error"] and
                                                           merrs[-1] <= GATE["posterior_mean_max_abs_error"])}}
    print(json.dumps(line), flush=True)


# DRAM bytes per sample of the streaming kernels, measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum) on the 12-round case of this
# workload and divided by the samples each launch processed: the append pass
# (550,000 retained samples) and the moments pass (600,000).
TRAFFIC_PER_SAMPLE = {"amis_append": 268.0, "moments": 265.7}
SPAN_SAMPLES = {"amis_append": lambda t, n: t * n, "moments": lambda t, n: (t + 1) * n}


def run_gb300(args):
    import torch

    rank, world, local_rank = dist_info()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local_rank if world > 1 else 0)
    torch.cuda.set_device(dev)
    import __graft_entry__ as ge

    issm = ge.load_package()
    issm.native.require()
    codes = {"fp32": issm.native.PREC_NATIVE, "tf32": issm.native.PREC_TF32, "bf16": issm.native.PREC_BF16}
    loc, L, p_loc, p_fac = problem()
    target = issm.StudentTTarget(loc, L, DOF)
    rounds, round_size = args.rounds, args.round_size
    total = rounds * round_size
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else (lambda: None)
    stream = torch.cuda.current_stream()

    def make(form):
        proposal = issm.FactorGaussian(p_loc.astype(np.float32), p_fac.astype(np.float32))
        alg = issm.AMIS(proposal, rounds=rounds, round_size=round_size)
        smp = issm.prepare_sampler(1234 + rank, target, alg, device=dev, precision=codes[form])
        smp.initial = tuple(t.clone() for t in smp.committed)

        def step():
            # each step restarts from the same initial proposal (no carried adaptation)
            for dst, src in zip(smp.committed, smp.initial):
                dst.copy_(src)
            return issm.importance_sample_(smp)
        return smp, step

    def measure(step, steps, warmup):
        """Time `steps` complete runs after `warmup` untimed ones. Every step
        already ends in one packed read of its failure words, summaries and
        posterior mean (the result's check), so its log Z and posterior
        mean are recorded per step at no extra device work."""
        for _ in range(warmup):
            res = step()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        l0 = issm.native.launches()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        logz, merr = [], []
        start.record(stream)
        for _ in range(steps):
            res = step()
            logz.append(float(res.diagnostics["round_lognormalizers"][-1]))
            merr.append(float(np.max(np.abs(res.diagnostics["moment_mean"] - loc))))
        end.record(stream)
        torch.cuda.synchronize()
        barrier()
        l1 = issm.native.launches()
        ms = start.elapsed_time(end) / steps
        if world > 1:
            t = torch.tensor([ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        signed = np.array(logz)
        lz = np.abs(signed)
        me = np.array(merr)
        se = float(signed.std(ddof=1) / np.sqrt(len(signed))) if len(signed) > 1 else float("nan")
        return {"ms": ms, "value": total * world / (ms / 1e3), "launches": int((l1 - l0) // steps),
                "logz_stats": {"mean_logz_hat": float(signed.mean()), "standard_error": se, "steps": len(signed)},
                "abs_logz_error": {"mean": float(lz.mean()), "max": float(lz.max()), "steps": len(lz)},
                "posterior_mean_max_abs_error": {"mean": float(me.mean()), "max": float(me.max())}}

    def same_draws(form, seed):
        """One fresh run of `form` from `seed` (its first call draws the
        first numbers of the seed's FP32 normal stream): per-round log Z."""
        proposal = issm.FactorGaussian(p_loc.astype(np.float32), p_fac.astype(np.float32))
        smp = issm.prepare_sampler(seed, target, issm.AMIS(proposal, rounds=rounds, round_size=round_size),
                                   device=dev, precision=codes[form])
        r = issm.importance_sample_(smp)
        out = np.asarray(r.diagnostics["round_lognormalizers"])
        del smp, r
        return out

    def fp64_same_draws(seed):
        """The FP64 form on the same draws as same_draws(form, seed): normals
        from the seed's FP32 stream and the FP32 ridge, so its fits differ
        from the reduced-precision runs' by arithmetic alone. Returns the
        completed sampler (for re-weighing) and its per-round log Z."""
        proposal = issm.FactorGaussian(p_loc, p_fac)
        smp = issm.prepare_sampler(seed, target, issm.AMIS(proposal, rounds=rounds, round_size=round_size),
                                   device=dev, precision=codes["fp32"], regularization=FP32_RIDGE)
        issm.share_normal_stream(smp, torch.float32)
        r = issm.importance_sample_(smp)
        return smp, np.asarray(r.diagnostics["round_lognormalizers"])

    def fp32_stream_normals(seed):
        """The normals a fresh sampler with `seed` draws in its first call
        (FP32 stream, offsets advanced by n d + 8 per round), as FP64 host
        data for the oracle."""
        parts, offset = [], 0
        for _ in range(rounds):
            n = round_size * D
            parts.append(issm.ops.fill_normals(n, torch.float32, dev, seed, offset).double().cpu().numpy())
            offset += n + 8
        return np.concatenate(parts)

    def divergence(a, b):
        """Per-round |d log Z| of two adaptive runs from the same draws."""
        dl = np.abs(a - b)
        within = int(np.argmax(dl > 1e-3)) if np.any(dl > 1e-3) else len(dl)
        return {"round1_abs_logz_diff": float(dl[0]), "final_abs_logz_diff": float(dl[-1]),
                "max_abs_logz_diff": float(dl.max()), "leading_rounds_within_1e-3": within}

    sampler, step = make(args.precision)
    warmup = max(args.warmup, 3)
    with ClockSampler(dev.index) as clocks:
        head = measure(step, args.steps, warmup)

    # per-kernel profile of one extra run: a spin kernel first lets the host
    # queue the whole run (about 600 launches and 600 events from Python), so
    # every span's events time only its kernels; the spin must outlast the
    # queueing or the later spans include host gaps
    # the spans come from the host round loop (a profiled run is not issued
    # natively): one unrecorded pass first creates its scratch buffers, since
    # a first allocation can synchronise the device and end the spin early
    sampler.profile = []
    step()
    torch.cuda.synchronize()
    sampler.profile = []
    torch.cuda._sleep(int(4e8))
    step()
    torch.cuda.synchronize()
    groups = {}
    for name, s0, s1, nbytes in sampler.profile:
        g = groups.setdefault(name, [0.0, 0, 0])
        g[0] += s0.elapsed_time(s1)
        g[1] += 1
        g[2] += nbytes
    sampler.profile = None
    dominant = max(groups, key=lambda k: groups[k][0])
    tms, cnt, nbytes = groups[dominant]
    hbm, tflops, src = read_peaks()
    achieved = (nbytes / cnt) / ((tms / cnt) / 1e3) / 1e9
    share = {k: round(v[0] / sum(x[0] for x in groups.values()), 4) for k, v in groups.items()}
    # every span against its own bound: HBM spans by their algorithmic bytes,
    # the prefix mixture (tensor-bound) by its algorithmic flops, d(d+1) per
    # (sample, component) pair (the triangular contraction), against the
    # measured burst bf16 rate (each launch is timed alone); the MMA flops it
    # issues (padded K, the bf16 x3 split, the full square) are given beside
    dp = 16 if D <= 16 else 32 if D <= 32 else 64
    split = 3 if args.precision == "bf16" else 1
    pairs = sum((t + 1) * round_size for t in range(rounds))
    alg_flops = pairs * D * (D + 1)
    mma_flops = pairs * 2 * dp * (dp + 16) * split
    kernels = {}
    for k, (ms, c, nb) in groups.items():
        if k == "mixture_new" and args.precision != "fp32":
            # the measured bf16 GEMM rate; tf32 MMAs run at half the bf16 rate
            peak = tflops if args.precision == "bf16" else tflops / 2
            ach = alg_flops / (ms / 1e3) / 1e12
            kernels[k] = {"bound": "tensor", "achieved": round(ach, 1), "peak": round(peak, 1), "unit": "TFLOP/s",
                          "frac": round(ach / peak, 4), "ms_per_run": round(ms, 3), "peak_kind": "burst",
                          "issued_mma_tflops": round(mma_flops / (ms / 1e3) / 1e12, 1)}
        elif k in ("draw", "target", "amis_append", "form_summary", "moments"):
            ach = nb / (ms / 1e3) / 1e9
            kernels[k] = {"bound": "hbm", "achieved": round(ach, 1), "peak": round(hbm, 1), "unit": "GB/s",
                          "frac": round(ach / hbm, 4), "ms_per_run": round(ms, 3)}
        else:
            kernels[k] = {"bound": "fp64 latency (one CTA per fit)", "ms_per_run": round(ms, 3)}
    traffic = None
    if dominant in TRAFFIC_PER_SAMPLE:
        samples = sum(SPAN_SAMPLES[dominant](t, round_size) for t in range(rounds) if dominant != "amis_append" or t > 0)
        traffic = TRAFFIC_PER_SAMPLE[dominant] * samples / cnt

    # the other forms on the same GPU, seed and workload, timed from the same
    # counter position as the headline (same warm-up count, graph capture
    # inside the warm-up)
    forms = {}
    if not args.quick:
        for form in ("fp32", "tf32", "bf16"):
            if form != args.precision:
                _, step_f = make(form)
                forms[form] = measure(step_f, min(args.steps, 10), warmup)
                del step_f
                torch.cuda.empty_cache()

    # matched accuracy against FP64 on the same draws. A whole adaptive run
    # amplifies any difference in a fit into the next round's draws (about
    # 2x per round here, heavy-tailed weights), so the arithmetic is compared
    # with the adaptation held fixed: every form re-weighs the FP64 run's 2M
    # samples under the FP64 run's own 40-slot history (frozen proposals).
    # The adaptive runs from the same draws are reported beside it, and the
    # FP64 oracle on the host cores (the CPU baseline) runs the same draws.
    same, cpu_value, cores, cpu_sample = {}, None, None, None
    if not args.quick:
        seed = 4242 + rank
        s64, logz64 = fp64_same_draws(seed)
        lz64, mean64, _ = issm.reweigh_amis(s64)
        frozen = {}
        for form in ("fp32", "tf32", "bf16"):
            lz, mean_f, _ = issm.reweigh_amis(s64, codes[form], torch.float32)
            frozen[form] = {"abs_logz_diff": abs(lz - lz64),
                            "posterior_mean_max_abs_diff": float(np.max(np.abs(mean_f - mean64)))}
        same = {"frozen_proposals_vs_fp64": frozen,
                "adaptive_vs_fp64": {form: divergence(same_draws(form, seed), logz64)
                                     for form in ("fp32", "tf32", "bf16")}}
        del s64
        torch.cuda.empty_cache()
        if rank == 0:
            normals = fp32_stream_normals(seed)
            secs, cores, out = oracle_amis(normals, round_size=round_size, rounds=rounds, regularization=FP32_RIDGE)
            del normals
            cpu_value = total / secs
            cpu_sample = (f"one complete run of the workload ({rounds} rounds x {round_size} samples, d=64), FP64 "
                          f"oracle AMIS on the draws of the same-draw comparison")
            same["adaptive_vs_fp64"]["fp64_oracle"] = divergence(np.asarray(out["round_logz"]), logz64)
            del out

    # e2e: host arrays in, summaries and posterior mean out, through the public API
    def e2e_step():
        tgt = issm.StudentTTarget(loc, L, DOF)
        prop = issm.FactorGaussian(p_loc.astype(np.float32), p_fac.astype(np.float32))
        smp = issm.prepare_sampler(99 + rank, tgt, issm.AMIS(prop, rounds=rounds, round_size=round_size),
                                   device=dev, precision=codes[args.precision])
        r = issm.importance_sample_(smp)
        pm = issm.mean(r).cpu().numpy()
        return r, pm

    # bytes copied per step: target location + scale factor and proposal
    # location + factor (float32) in; the run's packed read (per-round
    # failure words and summaries, the moment mean), the weight-sum word that
    # mean() checks and the posterior mean out
    h2d = (D + D * D) * 4 + (D + D * D) * 4
    d2h = rounds * 3 * 8 * 2 + D * 8 + 8 + D * 8
    e2e_ms = float("nan")
    if not args.quick:
        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        e2e_steps = max(2, args.steps // 2)
        for _ in range(e2e_steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    if rank != 0:
        return

    def gate(logz_err, mean_err):
        return bool(logz_err <= GATE["abs_logz_error"] and mean_err <= GATE["posterior_mean_max_abs_error"])

    acc = {
        "gate": GATE,
        # against the analytic target (log Z = 0, mean = location), every timed step
        "analytic": {"abs_logz_error": head["abs_logz_error"],
                     "posterior_mean_max_abs_error": head["posterior_mean_max_abs_error"],
                     "passes_gate": gate(head["abs_logz_error"]["max"], head["posterior_mean_max_abs_error"]["max"]),
                     "why": "Gaussian proposals against a nu=5 Student-t target have infinite-variance weights: "
                            "no form (FP64 included) reaches the analytic gate at 2M samples"},
        # the same draws in every form, against FP64 arithmetic on those draws
        "same_draws": same,
    }
    if same:
        fz = same["frozen_proposals_vs_fp64"]
        same["passes_gate"] = {form: gate(v["abs_logz_diff"], v["posterior_mean_max_abs_diff"])
                               for form, v in fz.items()}
        acc["abs_logz_diff_vs_fp64_same_draws"] = fz[args.precision]["abs_logz_diff"]
        acc["posterior_mean_diff_vs_fp64_same_draws"] = fz[args.precision]["posterior_mean_max_abs_diff"]
    # the estimator's own error, form by form, over the timed steps (different
    # draws each step): matched when the forms' mean log Zhat agree within
    # their standard errors
    acc["estimator_by_form"] = {args.precision: head["logz_stats"]}
    acc["estimator_by_form"].update({k: v["logz_stats"] for k, v in forms.items()})
    line = {
        "metric": METRIC, "value": head["value"], "unit": "weighted samples/s", "n_gpus": world,
        "steps": args.steps, "warmup": warmup, "ms_per_step": head["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "tf32": "tf32", "bf16": "bf16"}[args.precision],
        "data": "synthetic (seeded C4 inputs)",
        "config": {"workload": WORKLOAD if (rounds, round_size) == (ROUNDS, ROUND_SIZE) else
                   f"AMIS d=64, Student-t target (nu=5), {rounds} rounds x {round_size} samples (reduced case)",
                   "d": D, "rounds": rounds, "round_size": round_size,
                   "precision": args.precision + (" (bf16 x3 split)" if args.precision == "bf16" else ""),
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2: 512 MiB retained samples re-read every round"},
        "accuracy": acc,
        "forms": {k: {"value": v["value"], "ms_per_step": v["ms"], "steps": v["abs_logz_error"]["steps"],
                      "abs_logz_error": v["abs_logz_error"],
                      "posterior_mean_max_abs_error": v["posterior_mean_max_abs_error"],
                      "speedup_of_headline": head["value"] / v["value"]} for k, v in forms.items()},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_source": f"{src} hbm_gbs", "traffic": traffic,
                     "kernel_share": share, "kernels": kernels},
        "cpu_baseline": {"value": cpu_value, "unit": "weighted samples/s", "cores": cores, "kind": "port",
                         "sample": cpu_sample},
        "e2e": {"value": total * world / (e2e_ms / 1e3), "unit": "weighted samples/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
        "gpu_launches": head["launches"],
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def run_static_mis(args):
    """Static MIS microbench (seeded synthetic inputs): N = 4,194,304 samples,
    d = 16, a bank of K = 64 full-covariance Gaussians (mu ~ N(0, 4 I),
    Sigma = A A^T / d + 0.1 I with A ~ N(0, 1), L = chol(Sigma) in FP64,
    masses ~ Dirichlet(1)), a standard-normal target. One step: stratified
    assignment and draw, the balance-heuristic log q of every sample over all
    64 components (the tcgen05 mixture kernel, BF16 x3), the target, the log
    weights, their summary and normalisation, and systematic resampling of
    all N with one uniform plus the gather of the resampled samples. The
    mixture kernel's roofline uses its algorithmic flops N K d (d + 1)
    against the measured burst bf16 rate."""
    import torch

    import __graft_entry__ as ge

    issm = ge.load_package()
    issm.native.require()
    dev = torch.device("cuda", 0)
    n, d, k = 4_194_304, 16, 64
    rng = np.random.default_rng(2)
    props = []
    for _ in range(k):
        A = rng.normal(size=(d, d))
        L = np.linalg.cholesky(A @ A.T / d + 0.1 * np.eye(d))
        props.append(issm.FactorGaussian((2.0 * rng.normal(size=d)).astype(np.float32), L.astype(np.float32)))
    bank = issm.ProposalBank(props, rng.dirichlet(np.ones(k)).astype(np.float32))
    db = issm.pack(bank, dev)
    prec = {"fp32": issm.native.PREC_NATIVE, "tf32": issm.native.PREC_TF32, "bf16": issm.native.PREC_BF16}[args.precision]
    den = issm.ops.denominator(issm.native.DENOM_FULL, db.logmasses)
    target = issm.StandardNormalTarget(d).bind(dev, torch.float32)
    f32 = dict(dtype=torch.float32, device=dev)
    u = torch.empty(n, **f32)
    slots = torch.empty(n, dtype=torch.int32, device=dev)
    normals = torch.empty(n * d, **f32)
    x = torch.empty(n, d, **f32)
    lq, lt, lw, w = (torch.empty(n, **f32) for _ in range(4))
    anc = torch.empty(n, dtype=torch.int64, device=dev)
    xr = torch.empty(n, d, **f32)
    sm = torch.zeros(3, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    mix_ms = []

    def step(i, timed):
        issm.ops.fill_uniforms(n, torch.float32, dev, 77, 2 * i * n * (d + 1), out=u)
        issm.ops.static_assign(db.cdf, u, True, out=slots)
        issm.ops.fill_normals(n * d, torch.float32, dev, 78, 2 * i * n * (d + 1), out=normals)
        issm.ops.draw(db, normals, n, slots=slots, out=x)
        if timed:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        issm.ops.mixture_logdensity(db, den, x, precision=prec, out=lq)
        if timed:
            e1.record(stream)
            mix_ms.append((e0, e1))
        target.evaluate(x, out=lt, precision=prec)
        issm.ops.subtract_logweights(lt, lq, out=lw)
        issm.ops.logweight_summary(lw, out=sm)
        issm.ops.normalize(lw, sm, out=w)
        issm.ops.resample_systematic(lw, 0.5 / (i + 2), n, out=anc)
        issm.ops.gather(x, anc, out=xr)

    for i in range(max(args.warmup, 3)):
        step(i, False)
    torch.cuda.synchronize()
    l0 = issm.native.launches()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clocks:
        t0.record(stream)
        for i in range(args.steps):
            step(100 + i, True)
        t1.record(stream)
        torch.cuda.synchronize()
    launches = int((issm.native.launches() - l0) // args.steps)
    ms = t0.elapsed_time(t1) / args.steps
    mix = float(np.mean([a.elapsed_time(b) for a, b in mix_ms]))
    hbm, tflops, src = read_peaks()
    alg = n * k * d * (d + 1)
    achieved = alg / (mix / 1e3) / 1e12
    peak = tflops if args.precision == "bf16" else tflops / 2
    # parity of the mixture on a slice, against the FP64 oracle
    from oracle import oracle as orc

    sl = 4096
    ob = orc.BankView(d, orc.GAUSSIAN, orc.SCALE_FACTOR, db.locations.double().cpu().numpy(),
                      db.scales.double().cpu().numpy(), db.lognormalizers.double().cpu().numpy())
    xs = x[:sl].double().cpu().numpy()
    exp, _, _ = orc.mixture_logdensity(ob, xs.reshape(-1), orc.DENOM_FULL, db.logmasses.double().cpu().numpy())
    err = float(np.max(np.abs(lq[:sl].double().cpu().numpy() - exp) / np.maximum(1.0, np.abs(exp))))
    # CPU baseline: the oracle's mixture (all host cores) on a 1/16 slice
    cpu_n = n // 16
    xc = x[:cpu_n].double().cpu().numpy().reshape(-1)
    c0 = time.perf_counter()
    orc.mixture_logdensity(ob, xc, orc.DENOM_FULL, db.logmasses.double().cpu().numpy())
    cpu_s = time.perf_counter() - c0
    line = {"metric": "static MIS weighted samples/s", "value": n / (ms / 1e3), "unit": "weighted samples/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp32": "f32", "tf32": "tf32", "bf16": "bf16"}[args.precision], "data": "synthetic (seeded)",
            "config": {"workload": "static MIS, N=4,194,304, d=16, K=64 full-covariance Gaussians, stratified "
                                   "assignment, balance-heuristic denominator, normalise, systematic resampling",
                       "l2": "inputs larger than L2 (268 MB of samples)"},
            "mixture_kernel": {"ms": mix, "pairs_per_s": n * k / (mix / 1e3),
                               "max_rel_err_vs_fp64_oracle": err},
            "roofline": {"bound": "tensor", "kernel": "mixture_tc_kernel (K=64, BF16 x3)" if args.precision == "bf16"
                         else "mixture kernel", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "peak_source": f"{src} bf16_tflops (burst)",
                         "algorithmic_flops_per_launch": alg, "traffic": None},
            "cpu_baseline": {"value": cpu_n / cpu_s, "unit": "weighted samples/s (mixture density only)",
                             "cores": orc.num_threads(), "kind": "port",
                             "sample": f"FP64 oracle mixture density of {cpu_n} samples over the 64 components"},
            "gpu_launches": launches, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Serving mix (C5 shapes): independent Bayesian linear-regression
    posteriors, d ~ U{2..64}, n_obs log-uniform in [50, 5000], sample budget
    log-uniform in [1k, 100k] over 4 AMIS rounds, Poisson arrivals at each
    rate of the sweep; p50/p99 latency, retained weighted samples/s, and the
    worst errors against the conjugate analytic posteriors."""
    import torch

    import __graft_entry__ as ge

    issm = ge.load_package()
    issm.native.require()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(55)

    def make(count):
        reqs, truth = [], {}
        for rid in range(count):
            d = int(rng.integers(2, 65))
            n_obs = int(np.exp(rng.uniform(np.log(50), np.log(5000))))
            budget = int(np.exp(rng.uniform(np.log(1000), np.log(100_000))))
            X = rng.normal(size=(n_obs, d))
            beta = rng.normal(size=d)
            y = X @ beta + 0.5 * rng.normal(size=n_obs)
            tgt = issm.LinearRegressionTarget(X, y, sigma=0.5, prior_var=1.0)
            mean, logz = tgt.analytic()
            post_cov = np.linalg.inv(X.T @ X / 0.25 + np.eye(d))
            truth[rid] = (mean, np.sqrt(np.diag(post_cov)), logz)
            # warm start: the Laplace form displaced and widened by 0.5/sqrt(d) of its scale
            Lp = np.linalg.cholesky(post_cov)
            f = 0.5 / np.sqrt(d)
            p = issm.FactorGaussian((mean + f * Lp @ rng.normal(size=d)).astype(np.float32),
                                    ((1 + f) * Lp).astype(np.float32))
            reqs.append(issm.serving.ServeRequest(rid, tgt, p, rounds=4, round_size=max(budget // 4, 64),
                                                  seed=rid))
        return reqs, truth

    # warm-up: compile-free, but first launches and allocations
    prec = {"fp32": issm.native.PREC_NATIVE, "tf32": issm.native.PREC_TF32, "bf16": issm.native.PREC_BF16}[args.precision]
    grouped = args.serve_loop == "grouped"

    def loop():
        if grouped:
            return issm.serving.GroupedServeLoop(dev, max_inflight=args.inflight)
        return issm.serving.ServeLoop(dev, max_inflight=args.inflight, precision=prec)

    warm, _ = make(64)
    loop().run(warm)
    sweep = []
    for rate in args.rates:
        reqs, truth = make(args.requests)
        t = 0.0
        for r in reqs:
            t += rng.exponential(1.0 / rate)
            r.arrival = t
        launches0 = issm.native.launches()
        t0 = time.perf_counter()
        out = loop().run(reqs)
        wall = time.perf_counter() - t0
        launches = issm.native.launches() - launches0
        errors = sum(r.error is not None for r in out)
        out = [r for r in out if r.error is None]
        lat = np.array([r.latency for r in out])
        samples = sum(r.samples for r in reqs)
        lz = np.array([abs(r.logz - truth[r.rid][2]) for r in out])
        me = np.array([float(np.max(np.abs(r.posterior_mean - truth[r.rid][0]) / truth[r.rid][1])) for r in out])
        sweep.append({"rate_per_s": rate, "requests": len(reqs), "failed_runs": errors, "gpu_launches": launches,
                      "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                      "p99_ms": 1e3 * float(np.percentile(lat, 99)), "samples_per_s": samples / wall,
                      "runs_per_s": len(out) / wall, "wall_s": wall,
                      "abs_logz_error": {"p50": float(np.median(lz)), "p90": float(np.percentile(lz, 90)),
                                         "max": float(lz.max())},
                      "posterior_mean_error_sd": {"p50": float(np.median(me)), "p90": float(np.percentile(me, 90)),
                                                  "max": float(me.max())}})
    # CPU baseline: the FP64 oracle AMIS (OpenMP over samples) on a bounded
    # sample of the same mix, with fed normals
    from oracle import oracle as orc

    cpu_reqs, _ = make(args.cpu_requests)
    cpu_s, cpu_samples = 0.0, 0
    for r in cpu_reqs:
        t = r.target
        tv = orc.TargetView(orc.TARGET_LINREG, r.proposal.dimension, j=t.X.shape[0], a=t.X, b=t.y, p0=t.sigma,
                            p1=t.prior_var)
        normals = np.random.default_rng(r.rid).standard_normal(r.rounds * r.round_size * r.proposal.dimension)
        t0 = time.perf_counter()
        orc.amis_run(tv, r.proposal.dimension, r.proposal.location, r.proposal.factor_matrix(),
                     [r.round_size] * r.rounds, normals, regularization=float(np.sqrt(np.finfo(np.float32).eps)))
        cpu_s += time.perf_counter() - t0
        cpu_samples += r.rounds * r.round_size
    line = {"metric": "serving mix p50/p99 latency and weighted samples/s", "impl": "gb300",
            "workload": "Bayesian linear regression posteriors, d~U{2..64}, n_obs log-uniform 50-5000, "
                        "budget log-uniform 1k-100k, AMIS 4 rounds, Poisson arrivals; initial proposal the "
                        "posterior's Laplace form displaced and widened by 0.5/sqrt(d) of its scale",
            "serve_loop": args.serve_loop,
            "precision": ("fp32 (grouped SIMT kernels; compensated FP32 moment sums, FP64 merge and fit)" if grouped else
                          {"bf16": "bf16 (bf16 x3 split)", "tf32": "tf32", "fp32": "fp32"}[args.precision]),
            "max_inflight": args.inflight, "sweep": sweep,
            "cpu_baseline": {"runs_per_s": len(cpu_reqs) / cpu_s, "samples_per_s": cpu_samples / cpu_s,
                             "unit": "runs/s and weighted samples/s, back to back (no arrivals)",
                             "cores": orc.num_threads(), "kind": "port",
                             "sample": f"{len(cpu_reqs)} requests of the same mix, FP64 oracle AMIS on fed normals"}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--precision", default="bf16", choices=["fp32", "tf32", "bf16"],
                    help="bf16: the BF16 x3 tensor-core form (default); fp32: the plain FP32 drop-in form")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--rounds", type=int, default=ROUNDS)
    ap.add_argument("--round-size", type=int, default=ROUND_SIZE)
    ap.add_argument("--quick", action="store_true", help="skip the e2e and CPU-baseline legs (profiling runs)")
    ap.add_argument("--workload", default="amis", choices=["amis", "serve", "static-mis"],
                    help="amis: the headline AMIS d=64 run; serve: the serving-mix latency sweep; "
                         "static-mis: the N=4,194,304, d=16, K=64 static MIS microbench")
    ap.add_argument("--requests", type=int, default=10_000, help="serve: requests per arrival rate")
    ap.add_argument("--rates", type=float, nargs="+", default=[1000.0, 5000.0, 20000.0],
                    help="serve: arrivals per second")
    ap.add_argument("--cpu-requests", type=int, default=16, help="serve: requests in the CPU-baseline sample")
    ap.add_argument("--serve-loop", default="grouped", choices=["grouped", "streams"],
                    help="serve: grouped (one launch per phase per step for every in-flight run) or streams "
                         "(one issm_amis_run per run on its own stream)")
    ap.add_argument("--inflight", type=int, default=None,
                    help="serve: concurrent runs (default 4096 grouped, 8 streams)")
    args = ap.parse_args()
    if args.inflight is None:
        args.inflight = 4096 if args.serve_loop == "grouped" else 8
    if args.workload == "serve":
        run_serve(args)
        return
    if args.workload == "static-mis":
        run_static_mis(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
