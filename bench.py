#!/usr/bin/env python
"""Benchmark of the streaming LFMM2 fit on GB300: SNPs/s of one whole
fit_lfmm2 job (Step 0, the 2q+2 randomized-SVD passes, the association
pass with GIF calibration) on a synthetic cohort.

Default workload ("biobank"): n = 20,000 samples, p = 2,000,000 SNPs,
10 admixed populations (Dirichlet(0.3)), Fst 0.05, allele frequencies
U(0.01, 0.5), 0.5 % MCAR missing calls, 50 Gaussian traits jointly as
covariates (each with U(0, 30 %) of its values masked and mean-imputed the
way the reference CLI does), K = 20, oversampling 10, 2 power iterations.

Reported:
* ``value``  SNPs/s with the packed genotypes already resident in HBM;
* ``e2e``    SNPs/s through the C-ABI host entry point slfmm_fit_host:
             pinned host payload -> H2D -> fit -> results D2H, every step;
* ``roofline`` of the dominant contraction kernel (CUDA events, live);
* ``cpu_baseline`` the faithful n x n CPU restatement of the reference
             timed on a bounded SNP sample and extrapolated to p.

``--impl reference`` times only that CPU restatement (the reference crate
itself is Rust and cannot be built here).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SNPs/s end-to-end, split-FP8 vs FP32 GPU at max|Δt|≤1e-3; HBM/TC % of peak"

# batched workloads (not the headline): per-trait models on the biobank
# cohort, and many uneven independent problems
BATCHED = {
    # 50 traits, each its own d = 1 model on the samples where it is not masked
    # (U(0, 30 %) masked per trait), K = 20: the reference run once per trait
    # with --intersect-samples
    "traits": dict(n=20_000, p=2_000_000, k=20, traits=50, oversampling=10, power_iter=2, n_pop=10, alpha=0.3,
                   fst=0.05, f_lo=0.01, f_hi=0.5, miss=0.005, lam=1e-5, mask_max=0.3),
    # 64 independent problems: n ~ U[100, 3000], p ~ U[50k, 400k], K ~ U[2, 16],
    # 1-8 covariates, 2-6 populations with Fst ~ U(0.02, 0.2), 1 % MCAR
    "many": dict(problems=64, n_lo=100, n_hi=3000, p_lo=50_000, p_hi=400_000, k_lo=2, k_hi=16, d_lo=1, d_hi=8,
                 pop_lo=2, pop_hi=6, fst_lo=0.02, fst_hi=0.2, miss=0.01, streams=8),
}

WORKLOADS = {
    # the configuration the headline metric is quoted on
    "biobank": dict(n=20_000, p=2_000_000, k=20, d=50, oversampling=10, power_iter=2, n_pop=10, alpha=0.3,
                    fst=0.05, f_lo=0.01, f_hi=0.5, miss=0.005, inbreeding=0.0, lam=1e-5, mask_max=0.3,
                    est_rate=None),
    # same per-SNP shape on 100k SNPs (profiling slice, ~0.5 GB packed)
    "biobank-slice": dict(n=20_000, p=100_000, k=20, d=50, oversampling=10, power_iter=2, n_pop=10, alpha=0.3,
                          fst=0.05, f_lo=0.01, f_hi=0.5, miss=0.005, inbreeding=0.0, lam=1e-5, mask_max=0.3,
                          est_rate=None),
    # inbred-plant shape (parity/scale case)
    "plant": dict(n=1_135, p=1_800_000, k=12, d=1, oversampling=10, power_iter=2, n_pop=8, alpha=0.5,
                  fst=0.1, f_lo=0.01, f_hi=0.5, miss=0.02, inbreeding=0.9, lam=1e-5, mask_max=0.0,
                  est_rate=0.01),
    # NMF-imputation shape: 6 admixed populations, 7 % missing calls (MCAR here;
    # the 2 % contiguous-block share is drawn as MCAR too), nmf-k 8, 10 updates
    "nmf": dict(n=5_000, p=500_000, k=8, d=4, oversampling=10, power_iter=2, n_pop=6, alpha=0.4,
                fst=0.05, f_lo=0.01, f_hi=0.5, miss=0.07, inbreeding=0.0, lam=1e-5, mask_max=0.0,
                est_rate=None, nmf=dict(k=8, n_iter=10, cv_rate=5e-4)),
    # the reference's CPU-runnable case
    "small": dict(n=200, p=10_000, k=3, d=1, oversampling=10, power_iter=2, n_pop=2, alpha=1.0,
                  fst=0.1, f_lo=0.05, f_hi=0.5, miss=0.01, inbreeding=0.0, lam=1e-5, mask_max=0.0,
                  est_rate=None),
}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), float(d.get("bf16_tflops_sustained", d["bf16_tflops"])), "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


def traffic_from_profiles(kernel: str, workload: str):
    """dram bytes per launch from a committed ncu summary, if any."""
    f = ROOT / "profiles" / f"{kernel}_{workload}.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def make_covariates(n: int, d: int, q: np.ndarray, mask_max: float, seed: int) -> np.ndarray:
    """Gaussian traits with a population term; each trait has U(0, mask_max)
    of its values masked and imputed to the observed column mean, the way the
    reference CLI treats NA covariates (src/main.rs:543-568)."""
    rng = np.random.default_rng(seed)
    pop = q @ rng.normal(size=(q.shape[1], d))
    pop /= pop.std(axis=0) + 1e-12
    x = 0.4 * pop + rng.normal(size=(n, d))
    for t in range(d):
        frac = rng.uniform(0.0, mask_max) if mask_max > 0 else 0.0
        m = rng.random(n) < frac
        if m.any() and (~m).any():
            x[m, t] = x[~m, t].mean()
    return np.ascontiguousarray(x)


def pinned_empty(shape, dtype):
    import schnellfmm_gb300 as sg
    pa = sg.PinnedArray(shape, dtype)
    return pa.array, pa


def run_reference(args, w):
    """Time the CPU restatement of the reference on a bounded SNP sample."""
    from oracle import cpu_baseline, lfmm_oracle as O
    n, p = w["n"], w["p"]
    rng = np.random.default_rng(123)
    q = rng.dirichlet(np.full(w["n_pop"], w["alpha"]), size=n)
    x = make_covariates(n, w["d"], q, w["mask_max"], 7)
    sample = args.cpu_sample
    f_anc = rng.uniform(w["f_lo"], w["f_hi"], size=sample)
    sd = np.sqrt(w["fst"] * f_anc * (1 - f_anc))
    f_pop = np.clip(f_anc[None, :] + sd[None, :] * rng.normal(size=(w["n_pop"], sample)), 1e-3, 1 - 1e-3)
    g = rng.binomial(2, q @ f_pop).astype(np.int16)
    g[rng.random(g.shape) < w["miss"]] = 255
    packed = O.pack_codes(O.genotypes_to_codes(g.T))
    per_step = []
    info = None
    for it in range(args.warmup + args.steps):
        info = cpu_baseline.time_reference_cpu(packed, n, x, k=w["k"], oversampling=w["oversampling"],
                                               power_iter=w["power_iter"], lam=w["lam"], norm=O.NORM_EIGENSTRAT,
                                               p_total=p)
        if it >= args.warmup:
            per_step.append(info["snps_per_s"])
    return float(np.median(per_step)), info


def max_over_ranks(v: float, dist=None, device: str = "cpu") -> float:
    """Largest value over the replicas (the job's time is its slowest rank)."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: int, world: int, ms_max: float) -> float:
    """Whole-job throughput: the units every replica processed over the
    slowest replica's time."""
    return world * units_per_rank / (ms_max / 1e3)


def _event_ms(fn, steps, stream):
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) * 1e3 / steps
    return max(e0.elapsed_time(e1) / steps, wall)


def run_traits(args, w):
    """Per-trait models: one step = all traits of the cohort, each a full
    d = 1 fit on its own sample set (slfmm_fit_traits on the resident matrix).
    ``e2e`` adds the upload of the payload from pinned memory."""
    import torch
    import schnellfmm_gb300 as sg
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    eng = sg.Engine(0, sg.Precision.SPLIT_FP8, stream=stream.cuda_stream)
    n, p, t_count = w["n"], w["p"], w["traits"]
    rng = np.random.default_rng(100)
    q = rng.dirichlet(np.full(w["n_pop"], w["alpha"]), size=n).astype(np.float32)
    y = make_covariates(n, t_count, q.astype(np.float64), 0.0, 7)
    masks = np.ones((n, t_count), dtype=np.uint8)
    for t in range(t_count):
        masks[rng.random(n) < rng.uniform(0.0, w["mask_max"]), t] = 0
    geno = eng.simulate(q, p, fst=w["fst"], f_lo=w["f_lo"], f_hi=w["f_hi"], miss=w["miss"], seed=42)
    cfg = sg.Lfmm2Config(k=w["k"], lambda_=w["lam"], oversampling=w["oversampling"], n_power_iter=w["power_iter"],
                         norm=sg.SnpNorm.EIGENSTRAT)
    bps = (n + 3) // 4
    host_packed, _keep = pinned_empty((p, bps), np.uint8)
    geno.download(host_packed)
    for _ in range(args.warmup):
        sg.fit_lfmm2_traits(geno, y, masks, cfg, engine=eng)
    launches0 = eng.launches
    with ClockSampler(0) as clk:
        ms = _event_ms(lambda: sg.fit_lfmm2_traits(geno, y, masks, cfg, engine=eng), args.steps, stream)
    launches = (eng.launches - launches0) // max(args.steps, 1)

    def e2e_step():
        g = eng.upload(host_packed, n)
        sg.fit_lfmm2_traits(g, y, masks, cfg, engine=eng)
        g.free()
    e2e_step()
    ms_e2e = _event_ms(e2e_step, args.steps, stream)
    return {"metric": "SNPs/s per-trait LFMM2 (all traits of the cohort per step), split-FP8",
            "value": p / (ms / 1e3), "unit": "SNPs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "e4m3x4 split (exact e4m3 genotypes, fp32 accumulate)",
            "data": "synthetic (seeded structured cohort drawn on the device)",
            "config": {"workload": f"traits: n={n} p={p} K={w['k']} {t_count} traits x d=1, "
                                   f"U(0,{w['mask_max']}) of samples masked per trait",
                       "trait_sample_counts": [int(v) for v in masks.sum(axis=0)],
                       "l2": "inputs larger than L2 (packed genotypes %.1f GB)" % (p * bps / 1e9)},
            "trait_snps_per_s": p * t_count / (ms / 1e3),
            "e2e": {"value": p / (ms_e2e / 1e3), "unit": "SNPs/s", "h2d_bytes_per_step": int(p * bps),
                    "d2h_bytes_per_step": int(sum(p * 48 + int(m) * w["k"] * 8 for m in masks.sum(axis=0))),
                    "ms_per_step": ms_e2e},
            "gpu_launches": int(launches), "clocks": clk.summary()}


def run_many(args, w):
    """Many uneven independent problems: one step = all problems from pinned
    host payloads (upload, fit, results to pinned buffers), concurrently on
    several streams (slfmm_fit_many), against the same problems one at a time."""
    import torch
    import schnellfmm_gb300 as sg
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    eng = sg.Engine(0, sg.Precision.SPLIT_FP8, stream=stream.cuda_stream)
    rng = np.random.default_rng(500)
    problems, outs, keep, shapes = [], [], [], []
    h2d = d2h = 0
    for i in range(w["problems"]):
        n = int(rng.integers(w["n_lo"], w["n_hi"] + 1))
        p = int(rng.integers(w["p_lo"], w["p_hi"] + 1))
        k = int(rng.integers(w["k_lo"], w["k_hi"] + 1))
        d = int(rng.integers(w["d_lo"], w["d_hi"] + 1))
        n_pop = int(rng.integers(w["pop_lo"], w["pop_hi"] + 1))
        q = rng.dirichlet(np.full(n_pop, 0.5), size=n).astype(np.float32)
        g = eng.simulate(q, p, fst=float(rng.uniform(w["fst_lo"], w["fst_hi"])), f_lo=0.05, f_hi=0.5,
                         miss=w["miss"], seed=1000 + i)
        bps = (n + 3) // 4
        packed, t = pinned_empty((p, bps), np.uint8)
        g.download(packed)
        g.free()
        keep.append(t)
        x = make_covariates(n, d, q.astype(np.float64), 0.0, 2000 + i)
        cfg = sg.Lfmm2Config(k=k, oversampling=10, n_power_iter=2, seed=42 + i, norm=sg.SnpNorm.EIGENSTRAT)
        out = {}
        for name, shape in (("u_hat", (n, k)), ("beta", (p, d)), ("tstat", (p, d)), ("pvalue", (p, d)),
                            ("r2", (p, 3)), ("gif_per_trait", (d,))):
            a, ta = pinned_empty(shape, np.float64)
            out[name] = a
            keep.append(ta)
        problems.append((packed, n, x, cfg))
        outs.append(out)
        shapes.append((n, p, k, d))
        h2d += p * bps + x.nbytes
        d2h += sum(a.nbytes for a in out.values())
    total_snps = sum(s[1] for s in shapes)
    streams = w["streams"]
    for _ in range(args.warmup):
        sg.fit_lfmm2_many(problems, engine=eng, n_streams=streams, outs=outs)
    with ClockSampler(0) as clk:
        ms = _event_ms(lambda: sg.fit_lfmm2_many(problems, engine=eng, n_streams=streams, outs=outs), args.steps,
                       stream)

    def one_by_one():
        for (packed, n, x, cfg), out in zip(problems, outs):
            sg.fit_lfmm2_host(packed, n, x, cfg, engine=eng, out=out)
    one_by_one()
    ms_one = _event_ms(one_by_one, args.steps, stream)
    return {"metric": "aggregate SNPs/s over many uneven LFMM2 problems (host payloads), split-FP8",
            "value": total_snps / (ms / 1e3), "unit": "SNPs/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "e4m3x4 split (exact e4m3 genotypes, fp32 accumulate)",
            "data": "synthetic (seeded structured cohorts drawn on the device)",
            "config": {"workload": f"many: {len(problems)} problems, n U[{w['n_lo']},{w['n_hi']}], "
                                   f"p U[{w['p_lo']},{w['p_hi']}], K U[{w['k_lo']},{w['k_hi']}], "
                                   f"d {w['d_lo']}-{w['d_hi']}", "streams": streams, "total_snps": total_snps,
                       "l2": "inputs larger than L2 (%.1f GB of payloads)" % (h2d / 1e9)},
            "one_by_one": {"value": total_snps / (ms_one / 1e3), "unit": "SNPs/s", "ms_per_step": ms_one},
            "e2e": {"value": total_snps / (ms / 1e3), "unit": "SNPs/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": ms},
            "clocks": clk.summary()}


def _compare(res_t, res_beta, res_r2, ref) -> dict:
    """Per-SNP agreement of GPU results with an oracle AssocResults."""
    scale = float(np.abs(ref.beta).max()) or 1.0
    return {"max_abs_dt": float(np.abs(res_t - ref.tstat).max()),
            "max_abs_dbeta_over_max_beta": float(np.abs(res_beta - ref.beta).max() / scale),
            "max_abs_dr2": float(np.abs(res_r2 - ref.r2).max())}


def _top_overlap(t_gpu: np.ndarray, t_ref: np.ndarray, top: int = 100) -> float:
    """Smallest share, over traits, of the oracle's top-`top` |t| SNPs that
    are also in the GPU's top `top`."""
    worst = 1.0
    for j in range(t_ref.shape[1]):
        a = set(np.argsort(-np.abs(t_ref[:, j]))[:top].tolist())
        b = set(np.argsort(-np.abs(t_gpu[:, j]))[:top].tolist())
        worst = min(worst, len(a & b) / float(top))
    return worst


def link_probe(host_u8: np.ndarray, stream) -> dict:
    """Page-locked host<->device copy rates of this machine: 2 GB of the pinned
    payload to the device and back, as one copy each (CUDA events)."""
    import torch
    nbytes = int(min(host_u8.nbytes, 2 << 30))
    src = torch.from_numpy(host_u8.reshape(-1)[:nbytes])
    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for name, fn in (("h2d_gbs", lambda: dev.copy_(src, non_blocking=True)),
                     ("d2h_gbs", lambda: src.copy_(dev, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = nbytes / (e0.elapsed_time(e1) / 1e3) / 1e9
    del dev
    return out


def run_to_tsv(args, sg, eng, host_packed, n, x, cfg, est, out, p, d) -> dict:
    """The end-to-end path to the reference's output file: slfmm_fit_host
    from the page-locked payload, then <out>.tsv written and closed on local
    disk (coalesce_output_tsv's layout and "{:.6e}" numbers).  The .bim names
    are marshalled once, before timing; the file is deleted afterwards."""
    import ctypes
    import tempfile
    lib = sg.load_library()
    chrom = sg._CStrings(str(1 + j // 100_000) for j in range(p))
    sid = sg._CStrings(f"rs{j}" for j in range(p))
    names = sg._CStrings(f"trait{j}" for j in range(d))
    pos = np.ascontiguousarray(1000 + 10 * np.arange(p, dtype=np.uint64))
    r = sg._Results(None, sg._dptr(out["beta"]), sg._dptr(out["tstat"]), sg._dptr(out["pvalue"]),
                    sg._dptr(out["r2"]), None, 0.0, None, 0.0, 0.0, 0.0, 0)
    fd, path = tempfile.mkstemp(suffix=".tsv")
    os.close(fd)
    fit_ms, write_ms, size = [], [], 0
    try:
        for _ in range(args.tsv_steps):
            t0 = time.perf_counter()
            sg.fit_lfmm2_host(host_packed, n, x, cfg, est_subset=est, engine=eng, out=out)
            t1 = time.perf_counter()
            rc = lib.slfmm_write_tsv(path.encode(), p, d, chrom.arg(), pos.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                     sid.arg(), names.arg(), ctypes.byref(r), 0)
            t2 = time.perf_counter()
            if rc != 0:
                raise RuntimeError(f"slfmm_write_tsv failed ({rc})")
            fit_ms.append((t1 - t0) * 1e3)
            write_ms.append((t2 - t1) * 1e3)
        size = os.path.getsize(path)
    finally:
        os.remove(path)
    total = min(a + b for a, b in zip(fit_ms, write_ms))
    return {"value": p / (total / 1e3), "unit": "SNPs/s", "ms_per_step": total, "fit_host_ms": min(fit_ms),
            "write_tsv_ms": min(write_ms), "tsv_bytes": int(size), "steps": args.tsv_steps,
            "host_threads": os.cpu_count()}


def _nmf_parity(args, w, eng, cfg):
    """NMF imputation against the FP64 oracle on a slice of the NMF shape
    (all n samples, 20 000 SNPs of the same generator; the dense FP64 matrix
    of the full shape does not fit in host memory): per-iteration CV MAE of
    the estimation phase, the GWAS-phase CV, U_hat and the imputed fit's t."""
    import schnellfmm_gb300 as sg
    from oracle import lfmm_oracle as O
    n, d, k = w["n"], w["d"], w["k"]
    ps = 20_000
    rng = np.random.default_rng(301)
    q = rng.dirichlet(np.full(w["n_pop"], w["alpha"]), size=n).astype(np.float32)
    xsl = make_covariates(n, d, q.astype(np.float64), w["mask_max"], 19)
    g2 = eng.simulate(q, ps, fst=w["fst"], f_lo=w["f_lo"], f_hi=w["f_hi"], miss=w["miss"],
                      inbreeding=w["inbreeding"], seed=5151)
    pk = np.empty((ps, (n + 3) // 4), dtype=np.uint8)
    g2.download(pk)
    r = sg.fit_lfmm2(g2, sg.SubsetSpec.all(), g2, xsl, cfg, engine=eng)
    g2.free()
    raw = O.decode_raw(pk, n)
    nm = w["nmf"]
    ref = O.fit_oracle64(raw, raw, xsl, k=k, lam=w["lam"], oversampling=w["oversampling"],
                         power_iter=w["power_iter"], seed=cfg.seed, norm=O.NORM_EIGENSTRAT,
                         nmf=dict(k=nm["k"], n_iter=nm["n_iter"], eps=cfg.nmf.eps, cv_rate=nm["cv_rate"]),
                         chunk=cfg.chunk_size, rng=args.rng)
    out = _compare(r.tstat, r.beta, r.r2, ref.assoc)
    mae, mmae, cnt = ref.gwas_cv
    cv_gpu = np.asarray(r.nmf_cv, dtype=np.float64)
    cv_ref = np.asarray(ref.nmf.cv_mae_per_iter, dtype=np.float64)
    out.update({"workload": f"n={n} p={ps} K={k} d={d}, NMF k={nm['k']} x {nm['n_iter']} updates "
                            "(same generator, seed 5151)",
                "cv_mae_per_iter_gpu": cv_gpu.tolist(), "cv_mae_per_iter_oracle": cv_ref.tolist(),
                "cv_mae_max_rel_diff": float(np.max(np.abs(cv_gpu - cv_ref) / np.abs(cv_ref))),
                "gwas_cv_mae_gpu": float(r.nmf_gwas_cv_mae), "gwas_cv_mae_oracle": float(mae),
                "gwas_cv_count_gpu": int(r.nmf_gwas_cv_count), "gwas_cv_count_oracle": int(cnt),
                "sin_theta_u": O.principal_angles_sin_max(r.u_hat, ref.u_hat),
                "gif_gpu": float(r.gif), "gif_oracle": float(ref.assoc.gif)})
    return out


def run_parity(args, w, eng, geno_est, geno, est, host_packed, x, cfg):
    """Accuracy of the benchmarked configuration against the FP64 oracle
    (outside the timed region).

    * ``full``: one fit of the benchmarked matrix with host outputs; the
      oracle tests a fixed sample of 20 000 of its SNPs with the GPU's U_hat
      (the association pass at the full n, d and K), and the GIF of all p SNPs
      is recomputed from the GPU's t statistics by the oracle's histogram.
    * ``slice``: the same cohort generator at p = 100 000 SNPs, fitted end to
      end on the GPU (engine sketch stream) and by the oracle (same stream,
      streamed from the same packed matrix): U_hat subspace, t, beta, r2, GIF,
      top-100 overlap."""
    import schnellfmm_gb300 as sg
    from oracle import lfmm_oracle as O
    t0 = time.perf_counter()
    n, p, d, k = w["n"], w["p"], w["d"], w["k"]
    out = {"tolerance": {"max_abs_dt": 1e-3, "sin_theta_u": 1e-3}}
    if w.get("nmf") is not None:
        out["nmf_slice"] = _nmf_parity(args, w, eng, cfg)
        out["max_abs_dt"] = out["nmf_slice"]["max_abs_dt"]
        out["within_tolerance"] = bool(out["max_abs_dt"] <= 1e-3 and out["nmf_slice"]["sin_theta_u"] < 2e-3)
        out["oracle_seconds"] = time.perf_counter() - t0
        return out
    # the estimation matrix is already the subset upload when a rate is set
    res = sg.fit_lfmm2(geno_est, sg.SubsetSpec.all() if geno_est is not geno else est, geno, x, cfg, engine=eng)
    xs = O.center_covariates(x, False)
    pre = O.precompute_thin(xs, w["lam"])
    rs = np.random.default_rng(9)
    idx = np.sort(rs.choice(p, size=min(p, args.parity_snps), replace=False))
    ysub = O.PackedMatrix(np.asarray(host_packed), n, O.NORM_EIGENSTRAT, snps=idx)
    ref = O.assoc_oracle64_packed(ysub, xs, res.u_hat, pre.ridge_inv)
    full = _compare(res.tstat[idx], res.beta[idx], res.r2[idx], ref)
    hist = O.TsqHistogram(d)
    for s in range(0, p, 1 << 18):
        hist.add_chunk(res.tstat[s:s + (1 << 18)])
    gif_per, gif = hist.compute_gif()
    full.update({"snps_checked": int(len(idx)), "gif_gpu": float(res.gif), "gif_oracle_histogram": gif,
                 "max_abs_dgif_per_trait": float(np.abs(np.asarray(res.gif_per_trait) - gif_per).max())})
    out["full"] = full
    del res
    if w.get("nmf") is None and args.parity_slice_snps > 0:
        ps = args.parity_slice_snps
        rng = np.random.default_rng(300)
        q = rng.dirichlet(np.full(w["n_pop"], w["alpha"]), size=n).astype(np.float32)
        xsl = make_covariates(n, d, q.astype(np.float64), w["mask_max"], 17)
        g2 = eng.simulate(q, ps, fst=w["fst"], f_lo=w["f_lo"], f_hi=w["f_hi"], miss=w["miss"],
                          inbreeding=w["inbreeding"], seed=4242)
        pk = np.empty((ps, (n + 3) // 4), dtype=np.uint8)
        g2.download(pk)
        est_idx = O.subset_indices(ps, rate=w["est_rate"]) if w["est_rate"] else None
        g2e = eng.upload(pk, n, snps=sg.SubsetSpec.from_rate(w["est_rate"])) if w["est_rate"] else g2
        r2 = sg.fit_lfmm2(g2e, sg.SubsetSpec.all(), g2, xsl, cfg, engine=eng)
        l = k + w["oversampling"]
        omega = O.sketch_normal(args.rng, cfg.seed, n, l)
        ref2 = O.fit_oracle64_packed(pk, n, xsl, k=k, lam=w["lam"], oversampling=w["oversampling"],
                                     power_iter=w["power_iter"], norm=O.NORM_EIGENSTRAT, omega=omega,
                                     est_snps=est_idx)
        sl = _compare(r2.tstat, r2.beta, r2.r2, ref2.assoc)
        sl.update({"workload": f"n={n} p={ps} K={k} d={d} (same generator, seed 4242)",
                   "sin_theta_u": O.principal_angles_sin_max(r2.u_hat, ref2.u_hat),
                   "gif_gpu": float(r2.gif), "gif_oracle": float(ref2.assoc.gif),
                   "top100_overlap_min_over_traits": _top_overlap(r2.tstat, ref2.assoc.tstat)})
        out["slice"] = sl
        if g2e is not g2:
            g2e.free()
        g2.free()
    worst_dt = max(out["full"]["max_abs_dt"], out.get("slice", {}).get("max_abs_dt", 0.0))
    out["max_abs_dt"] = worst_dt
    out["within_tolerance"] = bool(worst_dt <= 1e-3 and out.get("slice", {}).get("sin_theta_u", 0.0) < 1e-3)
    out["oracle_seconds"] = time.perf_counter() - t0
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + sorted(BATCHED), default="biobank")
    ap.add_argument("--precision", choices=["split_fp8", "split_bf16", "fp32"], default="split_fp8")
    ap.add_argument("--cpu-sample", type=int, default=1000, help="SNPs in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32-path", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--out", default=None, help="also write the JSON line to this file")
    ap.add_argument("--autotune", action="store_true", help="let the engine tune its ring depths (warm-up does it)")
    ap.add_argument("--rng", choices=["counter", "chacha8"], default="chacha8",
                    help="random streams of the sketches and CV masks (chacha8: the reference's, the default)")
    ap.add_argument("--no-parity", action="store_true", help="skip the accuracy check against the FP64 oracle")
    ap.add_argument("--tsv-steps", type=int, default=1,
                    help="end-to-end steps that also write <out>.tsv to local disk (0: none)")
    ap.add_argument("--parity-snps", type=int, default=20_000, help="SNPs of the full fit checked by the oracle")
    ap.add_argument("--parity-slice-snps", type=int, default=100_000,
                    help="SNPs of the separately fitted slice checked end to end (0: none)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload in BATCHED:
        if rank == 0:
            line = (run_traits if args.workload == "traits" else run_many)(args, BATCHED[args.workload])
            print(json.dumps(line))
            if args.out:
                Path(args.out).write_text(json.dumps(line) + "\n")
        return
    w = WORKLOADS[args.workload]
    config = {"workload": f"{args.workload}: n={w['n']} p={w['p']} K={w['k']} d={w['d']} "
                          f"l={w['k'] + w['oversampling']} q={w['power_iter']}",
              "n_samples": w["n"], "n_snps": w["p"], "K": w["k"], "d": w["d"], "oversampling": w["oversampling"],
              "power_iter": w["power_iter"], "est_rate": w["est_rate"], "precision": args.precision,
              "autotune": bool(args.autotune), "rng": args.rng,
              "l2": "inputs larger than L2 (packed genotypes %.1f GB vs 129 MB L2)" % (w["p"] * ((w["n"] + 3) // 4) / 1e9)}

    if args.impl == "reference":
        if rank != 0:
            return
        val, info = run_reference(args, w)
        line = {"metric": METRIC, "impl": "reference", "value": val, "unit": "SNPs/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "cpu_baseline": {"value": val, "unit": "SNPs/s", "cores": info["cores"], "kind": "port",
                                 "sample": f"{info['sample_snps']} SNPs x {w['n']} samples through every pass of "
                                           f"the n x n CPU restatement, extrapolated to p={w['p']}"},
                "e2e": {"value": val, "unit": "SNPs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "detail": info}
        print(json.dumps(line))
        return

    import torch
    import schnellfmm_gb300 as sg

    dist = None
    if world > 1:
        import torch.distributed as td
        torch.cuda.set_device(local_rank)
        td.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
        dist = td
    else:
        torch.cuda.set_device(0)
    dev = local_rank if world > 1 else 0
    torch_stream = torch.cuda.current_stream()
    prec = {"split_fp8": sg.Precision.SPLIT_FP8, "split_bf16": sg.Precision.SPLIT_BF16,
            "fp32": sg.Precision.FP32}[args.precision]
    eng = sg.Engine(dev, prec, stream=torch_stream.cuda_stream, autotune=args.autotune,
                    rng=sg.SketchRng.CHACHA8 if args.rng == "chacha8" else sg.SketchRng.COUNTER)
    n, p, d, k = w["n"], w["p"], w["d"], w["k"]
    rng = np.random.default_rng(100 + rank)
    q = rng.dirichlet(np.full(w["n_pop"], w["alpha"]), size=n).astype(np.float32)
    x = make_covariates(n, d, q.astype(np.float64), w["mask_max"], 7 + rank)
    geno = eng.simulate(q, p, fst=w["fst"], f_lo=w["f_lo"], f_hi=w["f_hi"], miss=w["miss"],
                        inbreeding=w["inbreeding"], seed=42 + rank)
    cfg = sg.Lfmm2Config(k=k, lambda_=w["lam"], oversampling=w["oversampling"], n_power_iter=w["power_iter"],
                         norm=sg.SnpNorm.EIGENSTRAT)
    if w.get("nmf"):
        cfg.impute = sg.ImputeStrategy.NMF
        cfg.nmf = sg.NmfConfig(k=w["nmf"]["k"], n_iter=w["nmf"]["n_iter"], cv_rate=w["nmf"]["cv_rate"])
    est = sg.SubsetSpec.from_rate(w["est_rate"]) if w["est_rate"] else sg.SubsetSpec.all()
    bps = (n + 3) // 4
    host_packed, _keep_alive = pinned_empty((p, bps), np.uint8)
    geno.download(host_packed)
    geno_est = geno
    if w["est_rate"]:
        geno_est = eng.upload(host_packed, n, snps=est)

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def maxover(v):
        return max_over_ranks(v, dist, "cuda")

    def _fit_device_only(e):
        # slfmm_fit on the resident matrices with NULL host outputs: the whole
        # fit runs, results stay in device memory (no D2H)
        r = sg._Results(None, None, None, None, None, None, 0.0, None, 0.0, 0.0, 0.0, 0)
        c = cfg._c()
        e.check(e.lib.slfmm_fit(e.h, geno_est.h, geno.h, sg._ptr(x), d, ctypes.byref(c), None, ctypes.byref(r)))
        return r.gif

    # ---- resident (device) throughput ----
    for _ in range(args.warmup):
        _fit_device_only(eng)
    barrier()
    eng.profile(True)
    launches0 = eng.launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        barrier()
        ev0.record(torch_stream)
        for _ in range(args.steps):
            _fit_device_only(eng)
        ev1.record(torch_stream)
        barrier()
    ms_total = maxover(ev0.elapsed_time(ev1))
    launches = eng.launches - launches0
    prof = {kname: eng.profile_read(kname) for kname in ("row_contract", "col_contract", "assoc_epilogue", "row_fix", "cholqr2", "small_eigh", "small_inverse")}
    eng.profile(False)
    ms_step = ms_total / args.steps
    value = job_rate(p, world, ms_step)

    # ---- end-to-end through the host entry point ----
    e2e = None
    if not args.no_e2e:
        out = {}
        keep = []
        for name, shape in (("u_hat", (n, k)), ("beta", (p, d)), ("tstat", (p, d)), ("pvalue", (p, d)),
                            ("r2", (p, 3)), ("gif_per_trait", (d,))):
            a, t = pinned_empty(shape, np.float64)
            out[name] = a
            keep.append(t)
        for _ in range(args.warmup):
            sg.fit_lfmm2_host(host_packed, n, x, cfg, est_subset=est, engine=eng, out=out)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        calls = []
        t0 = time.perf_counter()
        e0.record(torch_stream)
        for _ in range(args.steps):
            tc = time.perf_counter()
            sg.fit_lfmm2_host(host_packed, n, x, cfg, est_subset=est, engine=eng, out=out)
            calls.append((time.perf_counter() - tc) * 1e3)
        e1.record(torch_stream)
        barrier()
        wall = (time.perf_counter() - t0) * 1e3 / args.steps
        e2e_ms = maxover(max(e0.elapsed_time(e1) / args.steps, wall))
        h2d = p * bps + (int(p * (w["est_rate"] or 0) + 1) * bps if w["est_rate"] else 0) + x.nbytes
        d2h = sum(a.nbytes for a in out.values())
        e2e = {"value": job_rate(p, world, e2e_ms), "unit": "SNPs/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
               "per_step_ms": [e0.elapsed_time(e1) / args.steps, wall], "call_wall_ms": calls,
               "call_wall_median_ms": statistics.median(calls)}
        # where one call's time goes (after the timed loop): device time per
        # phase from events on the engine's stream, host wall time per phase,
        # and this box's page-locked copy rates
        eng.profile(True)
        t0 = time.perf_counter()
        sg.fit_lfmm2_host(host_packed, n, x, cfg, est_subset=est, engine=eng, out=out)
        e2e["one_call_wall_ms"] = (time.perf_counter() - t0) * 1e3
        e2e["phases_of_one_call"] = eng.phases()
        eng.profile(False)
        e2e["link_probe"] = link_probe(host_packed, torch_stream)
        if args.tsv_steps > 0:
            e2e["to_tsv"] = run_to_tsv(args, sg, eng, host_packed, n, x, cfg, est, out, p, d)

    # ---- plain FP32 GPU path, same resident inputs ----
    fp32 = None
    if not args.no_fp32_path and prec != sg.Precision.FP32:
        eng32 = sg.Engine(dev, sg.Precision.FP32, stream=torch_stream.cuda_stream,
                          rng=sg.SketchRng.CHACHA8 if args.rng == "chacha8" else sg.SketchRng.COUNTER)
        _fit_device_only(eng32)
        barrier()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = max(1, min(3, args.steps))
        f0.record(torch_stream)
        for _ in range(reps):
            _fit_device_only(eng32)
        f1.record(torch_stream)
        barrier()
        ms32 = maxover(f0.elapsed_time(f1) / reps)
        fp32 = {"value": job_rate(p, world, ms32), "unit": "SNPs/s", "ms_per_step": ms32,
                "speedup_of_headline": ms32 / ms_step}
        if e2e is not None:
            # the same host-to-host call on the FP32 engine
            sg.fit_lfmm2_host(host_packed, n, x, cfg, est_subset=est, engine=eng32, out=out)
            barrier()
            t0 = time.perf_counter()
            f0.record(torch_stream)
            for _ in range(reps):
                sg.fit_lfmm2_host(host_packed, n, x, cfg, est_subset=est, engine=eng32, out=out)
            f1.record(torch_stream)
            barrier()
            ms32e = maxover(max(f0.elapsed_time(f1) / reps, (time.perf_counter() - t0) * 1e3 / reps))
            fp32["e2e"] = {"value": job_rate(p, world, ms32e), "unit": "SNPs/s", "ms_per_step": ms32e}
            fp32["e2e_speedup_of_headline"] = ms32e / e2e["ms_per_step"]
        eng32.close()

    # ---- roofline of the dominant kernel class ----
    hbm, bf16, bf16s, src = peaks()
    dom = max(("row_contract", "col_contract"), key=lambda kk: prof[kk]["ms"])
    pr = prof[dom]
    avg_ms = pr["ms"] / max(pr["launches"], 1)
    bytes_per = pr["bytes"] / max(pr["launches"], 1)
    flops_per = pr["flops"] / max(pr["launches"], 1)
    achieved_gbs = bytes_per / (avg_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
            "frac": achieved_gbs / hbm, "peak_source": src,
            "traffic": traffic_from_profiles(dom, args.workload),
            "avg_launch_ms": avg_ms, "launches": pr["launches"], "algorithmic_bytes_per_launch": bytes_per,
            "algorithmic_tflops": flops_per / (avg_ms / 1e3) / 1e12, "tensor_peak_tflops": bf16,
            "share_of_step": {kk: prof[kk]["ms"] / ms_total for kk in prof}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import cpu_baseline, lfmm_oracle as O  # noqa: F401
        s = min(args.cpu_sample, p)
        info = cpu_baseline.time_reference_cpu(np.asarray(host_packed[:s]), n, x, k=k, oversampling=w["oversampling"],
                                               power_iter=w["power_iter"], lam=w["lam"], norm=1, p_total=p)
        cpu = {"value": info["snps_per_s"], "unit": "SNPs/s", "cores": info["cores"], "kind": "port",
               "sample": f"first {s} SNPs x {n} samples of this workload through every pass of the n x n CPU "
                         f"restatement of the reference (numpy FP64), extrapolated to p={p}",
               "extrapolated_total_s": info["extrapolated_total_s"]}

    parity = None
    if rank == 0 and not args.no_parity:
        parity = run_parity(args, w, eng, geno_est, geno, est, host_packed, x, cfg)

    if rank == 0:
        line = {"metric": METRIC, "value": value,
                "value_kind": "resident: packed genotypes already in HBM when the timed region starts "
                              "(the host-to-host number through the C ABI is e2e)",
                "unit": "SNPs/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": {sg.Precision.SPLIT_FP8: "e4m3x4 split (exact e4m3 genotypes, fp32 accumulate)",
                          sg.Precision.SPLIT_BF16: "bf16x2 split (exact bf16 genotypes, fp32 accumulate)",
                          sg.Precision.FP32: "fp32"}[prec],
                "data": "synthetic (seeded structured cohort drawn on the device)",
                "config": config, "e2e": e2e, "gpu_launches": int(launches), "roofline": roof,
                "cpu_baseline": cpu, "fp32_gpu_path": fp32, "parity": parity, "clocks": clk.summary()}
        s = json.dumps(line)
        print(s)
        if args.out:
            Path(args.out).write_text(s + "\n")
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
