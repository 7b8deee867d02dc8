#!/usr/bin/env python
"""Headline benchmark of the GB300 sumcheck prover.

Workload: InnerProductProver (MSB), num_vars = 26 -- two tables of 2^26
seeded uniform Goldilocks values (512 MiB each) -- with Fp3 challenges from
the Keccak device transcript; 26 rounds + finalize + final value, the whole
protocol on the device, replayed as one CUDA graph per proof.

One step = one proof.  `value` is input evaluations per second
(2 * 2^26 per proof) with the tables resident in HBM; `e2e` is the same
metric through the C ABI from pinned host buffers (H2D of both tables inside
the step, D2H of the proof).  The inputs (1 GiB) are larger than L2, so no
flush runs between steps.

`--impl reference` times the CPU implementation of the same path (the C
restatement in oracle/, all host threads; the Rust reference crate cannot be
built here) on the same workload and metric.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

# The CPU baselines run the oracle's OpenMP loops in this process; with
# threads that spin after each parallel region they compete with the host
# thread that launches the next GPU workload's graphs (Multilinear n = 20,
# launched right after the headline's CPU baseline, measured 180 against
# 169 us per proof).  Idle OpenMP threads sleep instead.
os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "efficient-sumcheck_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

SEED = 0x5EED_2026
LABEL = b"effsc-gpu/ip/v1"
METRIC = "evals/s"
UNIT = "evals/s"


# DRAM bytes per launch of the dominant kernel, from an ncu capture of this
# bench at full size (dram__bytes_read.sum + dram__bytes_write.sum averaged
# over the kernel's launches in one proof); keyed by (kernel, num_vars).
# DRAM bytes (read + write) per launch of each pass at num_vars = 26, from
# one full-size ncu capture of dram__bytes_read.sum / dram__bytes_write.sum
# (a one-pass metric set) of `bench.py --only inner_product_msb --num-vars 26
# --steps 1`; the fused rounds' figure is the average over their launches.
NCU_TRAFFIC = {("ip_round_3_triple_fold", 26): 1449.9e6, ("ip_rounds_0_2", 26): 1077.2e6,
               ("fused_round_fp3", 26): 144.4e6}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--num-vars", type=int, default=26)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--batch-instances", type=int, default=512,
                    help="batching leg: this many IP instances, num_vars uniform on 10..=22 (0 = skip)")
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other single-proof workloads (Multilinear n=20, Coefficient / EqFactored "
                         "n=24, GKR k=12, InnerProduct LSB n=26, host-resident n=28, ProtoGalaxy fold)")
    ap.add_argument("--serve-requests", type=int, default=20000,
                    help="serving leg: this many requests, 70%% IP / 30%% ML, num_vars uniform on 14..=26 (0 = skip)")
    ap.add_argument("--serve-slots", type=int, default=128)
    ap.add_argument("--serve-host-requests", type=int, default=2000,
                    help="requests of the host-fed serving leg (tables in pinned host memory)")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--only", choices=["protogalaxy_fold", "multilinear_n20", "gkr_k12", "inner_product_msb",
                                       "inner_product_lsb", "coefficient_eqfg"],
                    help="run one workload alone and print its record (for profiling); the last three run "
                         "--steps proofs at --num-vars without a CUDA graph, one launch per kernel")
    return ap.parse_args()


def config(n_vars, world, impl="ours"):
    how = ("whole protocol on the device, replayed as one CUDA graph" if impl == "ours"
           else "CPU implementation, all host threads")
    return {
        "workload": "InnerProductProver MSB, num_vars=%d: a, b = 2^%d seeded uniform Goldilocks "
                    "values each, Fp3 challenges from the Keccak transcript, %d rounds + "
                    "finalize; %s" % (n_vars, n_vars, n_vars, how),
        "num_vars": n_vars,
        "tables": 2,
        "challenge_field": "Fp3 (F64Ext3)",
        "transcript": "Keccak-f[1600] duplex, label %s" % LABEL.decode(),
        "l2": "inputs (2 x %d MiB) larger than L2 (129 MB); no flush" % ((8 << n_vars) >> 20),
        "parallelism": "replicas x%d" % world,
    }


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return []
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = []
        for line in out.splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append({"sm": float(parts[1]), "max": float(parts[2]), "power": float(parts[3]),
                             "hw": parts[5], "hwt": parts[6], "swt": parts[7], "pcap": parts[8]})
            except ValueError:
                continue
        return rows


def summarize_clocks(rows):
    if not rows:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
    busy = [r for r in rows if r["power"] > 300] or rows
    reasons = set()
    for r in busy:
        if r["hw"].lower().startswith("active"):
            reasons.add("hw_slowdown")
        if r["hwt"].lower().startswith("active"):
            reasons.add("hw_thermal_slowdown")
        if r["swt"].lower().startswith("active"):
            reasons.add("sw_thermal_slowdown")
        if r["pcap"].lower().startswith("active"):
            reasons.add("sw_power_cap")
    return {"sm_mhz": statistics.median(r["sm"] for r in busy), "sm_max_mhz": max(r["max"] for r in rows),
            "reasons": sorted(reasons), "samples": len(busy), "power_w_max": max(r["power"] for r in rows)}


# ---------------------------------------------------------------------------
# reference arm: the CPU implementation, all host threads
# ---------------------------------------------------------------------------
def cpu_proof_seconds(n_vars, check_against=None):
    """One oracle IP proof at num_vars; returns (seconds, proof)."""
    from oracle import oracle as O
    n = 1 << n_vars
    a = O.gen_table(O.table_seed(SEED, 0), n)
    b = O.gen_table(O.table_seed(SEED, 1), n)
    pr = O.Prover(O.IP, O.MSB, 3, [a, b])
    t0 = time.perf_counter()
    rp, ch, fv = O.sumcheck(pr, n_vars, O.Transcript(3, label=LABEL))
    dt = time.perf_counter() - t0
    return dt, (rp, ch, fv)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    n_vars = args.num_vars
    # bound a step to a few seconds: calibrate on a smaller case first
    probe = min(n_vars, 20)
    dt, _ = cpu_proof_seconds(probe)
    est = dt * (1 << (n_vars - probe))
    sample_vars = n_vars
    while est > 8.0 and sample_vars > 16:
        sample_vars -= 1
        est /= 2
    times = []
    for i in range(args.warmup + args.steps):
        dt, _ = cpu_proof_seconds(sample_vars)
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = args.steps * 2 * (1 << sample_vars) / total
    cfg = config(n_vars, args.gpus, "reference")
    if sample_vars != n_vars:
        # a slower host: the steps ran a smaller proof; say so in the config
        cfg["num_vars"] = sample_vars
        cfg["workload_num_vars"] = n_vars
        cfg["workload"] += " (this host ran num_vars=%d per step to bound the run)" % sample_vars
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64 (Goldilocks Fp / Fp3)", "data": "synthetic: seeded uniform Goldilocks tables",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "full protocol (IP MSB, Fp3 challenges, Keccak transcript) at "
                                   "num_vars=%d per step; C restatement of the reference algorithms "
                                   "(oracle/), not the Rust reference binary" % sample_vars},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import numpy as np
    import torch
    import effsc_gpu as E
    from effsc_gpu import _lib

    from effsc_gpu.replicas import Replicas, job_rate, replica_seed
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    rep = Replicas()
    world, rank = rep.world, rep.rank
    barrier = rep.barrier

    L = E.load()
    ctx = E.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    n_vars = args.num_vars
    n = 1 << n_vars

    # inputs generated on the device (seeded), resident in HBM
    a_dev = torch.empty(n, dtype=torch.int64, device="cuda")
    b_dev = torch.empty(n, dtype=torch.int64, device="cuda")
    seed = replica_seed(SEED, rank)
    for t, buf in enumerate((a_dev, b_dev)):
        _lib.check(L.effsc_gen_uniform(ctx.h, E.table_seed(seed, t), n,
                                       _lib.ctypes.cast(_lib.ctypes.c_void_p(buf.data_ptr()), _lib.u64p), None))
    prover = E.InnerProductProver.from_device([a_dev.data_ptr(), b_dev.data_ptr()], [n, n], [1, 1], field=E.FP3, ctx=ctx)

    def one_proof(use_graph=True):
        prover.reset()
        return prover.prove(n_vars, E.Transcript.keccak(E.FP3, LABEL), use_graph=use_graph)

    for _ in range(max(args.warmup, 3)):
        one_proof()
    torch.cuda.synchronize()

    # ---- timed region (device-resident inputs) ----
    sampler = ClockSampler(local)
    sampler.start()
    E.launch_count_reset()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    w0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        proof = one_proof()
    ev1.record(stream)
    barrier()
    wall = time.perf_counter() - w0
    launches = E.launch_count()
    ms = ev0.elapsed_time(ev1)
    # keep the GPU busy a little longer if the timed region was too short to sample clocks
    extra = 0
    t_end = time.perf_counter() + 1.5
    while wall < 1.5 and time.perf_counter() < t_end:
        one_proof()
        extra += 1
    torch.cuda.synchronize()
    clocks = summarize_clocks(sampler.stop())
    if extra:
        clocks["sampled_during"] = "timed region + %d more identical steps" % extra
    ms = rep.max(ms)
    evals_per_step = 2 * n
    value = job_rate(evals_per_step, args.steps, world, ms)

    # ---- per-kernel timing (one proof outside the graph) -> roofline ----
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs") or 6800.0
    peak_src = "measured" if peaks.get("hbm_gbs") else "fallback"
    L.effsc_profile_clear()
    L.effsc_profile_enable(1)
    one_proof(use_graph=False)
    L.effsc_profile_enable(0)
    torch.cuda.synchronize()
    per = {}
    nrec = L.effsc_profile_count()
    for i in range(nrec):
        name = _lib.ctypes.create_string_buffer(64)
        msv = _lib.ctypes.c_double()
        by = _lib.ctypes.c_uint64()
        _lib.check(L.effsc_profile_get(i, name, 64, _lib.ctypes.byref(msv), _lib.ctypes.byref(by)))
        k = name.value.decode()
        d = per.setdefault(k, {"launches": 0, "ms": 0.0, "bytes": 0})
        d["launches"] += 1
        d["ms"] += msv.value
        d["bytes"] += by.value
    L.effsc_profile_clear()
    dom = max(per, key=lambda k: per[k]["ms"])
    d = per[dom]
    achieved = d["bytes"] / (d["ms"] * 1e-3) / 1e9
    kernel_ms = sum(v["ms"] for v in per.values())
    alg_bytes_proof = sum(v["bytes"] for v in per.values())
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": NCU_TRAFFIC.get((dom, n_vars)),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, full-size capture"
                                  if (dom, n_vars) in NCU_TRAFFIC else None,
                "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs, burst copy)",
                "launches_per_proof": d["launches"], "bytes_per_launch_avg": d["bytes"] / d["launches"],
                "ms_per_launch_avg": d["ms"] / d["launches"]}
    mm = _lib.ctypes.c_double()
    f3 = _lib.ctypes.c_double()
    _lib.check(L.effsc_diag_mulmod_rate(ctx.h, _lib.ctypes.byref(mm), _lib.ctypes.byref(f3)))
    mac = _lib.ctypes.c_double()
    red = _lib.ctypes.c_double()
    _lib.check(L.effsc_diag_accumulate_rate(ctx.h, _lib.ctypes.byref(mac), _lib.ctypes.byref(red)))
    prods, reds = ip_fp3_ops_as_run(n_vars)
    ms_proof = ms / args.steps
    int_roof_ms = (prods / mac.value + reds / red.value) * 1e3
    hbm_roof_ms = alg_bytes_proof / (hbm_peak * 1e9) * 1e3

    # ---- e2e through the C ABI from pinned host buffers ----
    a_host = torch.empty(n, dtype=torch.int64, pin_memory=True)
    b_host = torch.empty(n, dtype=torch.int64, pin_memory=True)
    a_host.copy_(a_dev.cpu())
    b_host.copy_(b_dev.cpu())
    an = a_host.numpy().view(np.uint64)
    bn = b_host.numpy().view(np.uint64)

    def e2e_step():
        pr = E.InnerProductProver(an, bn, field=E.FP3, ctx=ctx)
        pf = pr.prove(n_vars, E.Transcript.keccak(E.FP3, LABEL), use_graph=False)
        del pr
        return pf

    def e2e_step_in_place():
        # the same tables read in place by the first pass over the host link,
        # which also copies them to the device for the second pass
        pr = E.InnerProductProver.from_host([an, bn], field=E.FP3, ctx=ctx)
        pf = pr.prove(n_vars, E.Transcript.keccak(E.FP3, LABEL), use_graph=False)
        del pr
        return pf

    def time_e2e(step):
        step()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.e2e_steps):
            pf = step()
        e1.record(stream)
        barrier()
        assert (pf.round_polys == proof.round_polys).all(), "e2e proof differs from the device-resident proof"
        return rep.max(e0.elapsed_time(e1)), pf

    e2e_copy_ms, pf_e2e = time_e2e(e2e_step)
    e2e_inplace_ms, pf_e2e = time_e2e(e2e_step_in_place)
    e2e_ms = min(e2e_copy_ms, e2e_inplace_ms)
    e2e_path = ("effsc_prover_create_host (pinned host tables read in place by the first pass, which copies them "
                "to the device) + effsc_prove + proof D2H" if e2e_inplace_ms <= e2e_copy_ms else
                "effsc_prover_create (pinned host tables copied to the device) + effsc_prove + proof D2H")
    e2e_value = job_rate(evals_per_step, args.e2e_steps, world, e2e_ms)
    proof_words = n_vars * 2 * 3 + n_vars * 3 + 3
    d2h = 8 * proof_words + 216 + 2 * 24
    assert (pf_e2e.round_polys == proof.round_polys).all(), "e2e proof differs from the device-resident proof"

    # ---- CPU baseline (rank 0, N=1) and full-size bit-exactness ----
    cpu = None
    bit_exact = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        cores = os.cpu_count() or 1
        O.set_threads(cores)
        pr_o = O.Prover(O.IP, O.MSB, 3, [an, bn])
        t0 = time.perf_counter()
        rp, ch, fv = O.sumcheck(pr_o, n_vars, O.Transcript(3, label=LABEL))
        dt = time.perf_counter() - t0
        bit_exact = bool((rp == proof.round_polys).all() and (ch == proof.challenges).all()
                         and (fv == proof.final_value).all())
        cpu = {"value": 2 * n / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "one full proof at num_vars=%d (same inputs and transcript), %.1f s; C restatement "
                         "of the reference algorithms (oracle/), not the Rust binary" % (n_vars, dt)}
        assert bit_exact, "GPU proof differs from the oracle at full size"

    configs = None
    if not args.no_configs and world == 1:
        configs = run_configs(args, E, L, ctx, stream, rank)
    batch = None
    if args.batch_instances and world == 1:
        batch = run_batch(args, E, L, ctx, stream, rank)
    serving = None
    if args.serve_requests and world == 1:
        serving = run_serving(args, E, ctx)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_proof, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64 (Goldilocks Fp / Fp3, exact modular)",
            "data": "synthetic: seeded uniform Goldilocks tables (SplitMix64), generated on device",
            "config": config(n_vars, world),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_ms / args.e2e_steps, "path": e2e_path,
                    "ms_per_step_by_path": {"create_copy": e2e_copy_ms / args.e2e_steps,
                                            "create_host_read_in_place": e2e_inplace_ms / args.e2e_steps}},
            "gpu_launches": launches,
            "clocks": clocks,
            "hbm_gbs_per_sumcheck": alg_bytes_proof / (ms_proof * 1e-3) / 1e9,
            "algorithmic_bytes_per_proof": alg_bytes_proof,
            "kernel_ms_per_proof": kernel_ms,
            "int_roofline": {"accumulate_products_per_s": mac.value, "reductions_per_s": red.value,
                             "products_as_run": prods, "reductions_as_run": reds, "roofline_ms": int_roof_ms,
                             "peak_source": "effsc_diag_accumulate_rate: independent lazy sums (the kernels' "
                                            "accumulate form) and 160-bit reductions, each on a full grid",
                             "counting": "64 x 64-bit products and reductions of the algorithm as run "
                                         "(ip_fp3_ops_as_run); roofline_ms = products / rate + reductions / rate",
                             "lower_rate_gl_mul_chains_per_s": mm.value,
                             "lower_rate_note": "a product with a full reduction each (gl_mul chains); the kernels "
                                                "never reduce per product, so this is not the peak",
                             "fp3_mul_per_s": f3.value},
            "hbm_roofline_ms": hbm_roof_ms,
            "one_pass_per_round_equivalent": {
                "algorithmic_bytes": 128 * n, "algorithmic_mulmods": 20 * n,
                "equivalent_gbs": 128 * n / (ms_proof * 1e-3) / 1e9,
                "note": "textbook schedule (one fold+evaluate pass per round), for comparison only: the proof "
                        "computes rounds 0-3 in two passes over the base tables and moves 56N bytes, so this is "
                        "not its roofline"},
            "frac_of_lower_roofline": max(hbm_roof_ms, int_roof_ms) / ms_proof,
            "per_kernel": {k: {"launches": v["launches"], "ms": round(v["ms"], 4),
                               "GB/s": v["bytes"] / (v["ms"] * 1e-3) / 1e9 if v["ms"] else None}
                           for k, v in per.items()},
            "bit_exact_vs_oracle": bit_exact,
            "other_workloads": configs,
            "batching": batch,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    rep.close()


# ---------------------------------------------------------------------------
# batching: a cohort of IP instances of uneven size
# ---------------------------------------------------------------------------
BATCH_SEED = 0xBA7C_2026


def batch_workload(count):
    """num_vars uniform on 10..=22 and per-instance table seeds, all seeded."""
    import random
    rng = random.Random(BATCH_SEED)
    nv = [rng.randint(10, 22) for _ in range(count)]
    return nv


def batch_label(i):
    return ("effsc-gpu/batch/%d" % i).encode()


def ip_fp3_ops_as_run(n_vars):
    """64 x 64-bit products and 160-bit -> canonical reductions of one IP MSB
    proof over Fp3 challenges as the device runs it (base tables of 2^n_vars,
    n_vars >= 14): the first pass, 26 products per octet (N/8 octets, its
    sums reduced once per thread); the triple fold, per item (two octets of
    both tables, N/16 items) 4 x 21 products for the folds and 18 for round
    3's two Fp3 x Fp3 sums, 12 reductions (the folded entries); every later
    round (and the tail's rounds), per quadruple of the table being folded,
    4 Fp3 folds of 9 products and 2 Fp3 x Fp3 sums of 9, 12 reductions."""
    N = 1 << n_vars
    prods = 26 * (N // 8) + (4 * 21 + 18) * (N // 16)
    reds = 12 * (N // 16)
    L = N // 8
    while L >= 4:
        prods += 54 * (L // 4)
        reds += 12 * (L // 4)
        L //= 2
    return prods, reds


def ip_fp3_bytes_as_run(n_vars):
    """Algorithmic HBM bytes of one IP MSB proof over Fp3 challenges as the
    batched path runs it without the tail: rounds 0-1 read both base tables
    (16 B per entry), round 2 reads them again and writes the Fp3 tables of
    length N/4 (16 + 12 B per entry), round r >= 3 reads the Fp3 tables of
    length N / 2^(r-1) and writes the halves (72 B per input entry);
    num_vars < 3 runs one pass per round."""
    if n_vars < 3:
        return ip_fp3_bytes(n_vars)
    N = 1 << n_vars
    tot = 16 * N + 28 * N
    for r in range(3, n_vars):
        tot += 72 * (N >> (r - 1))
    return tot + 96


def ip_fp3_bytes(n_vars):
    """Algorithmic HBM bytes of one IP MSB proof over Fp3 challenges (base
    tables of 2^n_vars): round 0 reads both base tables; round 1 reads them
    again and writes Fp3 halves; round k >= 2 reads the Fp3 tables of length
    2^(n-k+1) and writes the halves; finalize reads 2 x 2 Fp3 values."""
    N = 1 << n_vars
    tot = 16 * N
    for k in range(1, n_vars):
        lin = N >> (k - 1)
        tot += (16 if k == 1 else 48) * lin + 24 * lin
    return tot + 96


def run_batch(args, E, L, ctx, stream, rank):
    import numpy as np
    import torch
    count = args.batch_instances
    nv = batch_workload(count)
    seeds = [[E.table_seed(BATCH_SEED + i, t) for t in range(2)] for i in range(count)]
    b = E.Batch(E.IP, nv, seeds=seeds, field=E.FP3, ctx=ctx)
    txs = lambda: [E.Transcript.keccak(E.FP3, batch_label(i)) for i in range(count)]  # noqa: E731
    cache = os.path.join(PKG, "_build", "autotune.jsonl")
    q, tail = b.tune(txs(), cache_path=cache)
    tune_rec = None
    try:
        tune_rec = json.loads(open(cache).read().strip().splitlines()[-1])
    except (OSError, ValueError, IndexError):
        pass
    # batched: one graph replay per cohort, proofs copied back every step
    for _ in range(3):
        batch_out = b.prove_raw(txs())
    torch.cuda.synchronize()
    tx_sets = [txs() for _ in range(args.batch_steps)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.batch_steps):
        batch_out = b.prove_raw(tx_sets[k])
    e1.record(stream)
    torch.cuda.synchronize()
    ms_batch = e0.elapsed_time(e1) / args.batch_steps
    rp, ch, fv = batch_out
    rows = np.concatenate([[0], np.cumsum(nv)])

    # one at a time: a solo prover per instance on the same device tables,
    # each proof replayed from its own graph (captured during warm-up)
    solos = []
    for i in range(count):
        ptrs = [b.device_table(i, t) for t in range(2)]
        solos.append(E.InnerProductProver.from_device(ptrs, [1 << nv[i]] * 2, [1, 1], field=E.FP3, ctx=ctx))

    def solo_all():
        out = []
        for i, p in enumerate(solos):
            p.reset()
            out.append(p.prove(nv[i], E.Transcript.keccak(E.FP3, batch_label(i))))
        return out

    solo_all()
    torch.cuda.synchronize()
    steps1 = max(1, args.batch_steps // 2)
    e0.record(stream)
    for _ in range(steps1):
        solo_out = solo_all()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_solo = e0.elapsed_time(e1) / steps1
    same_as_solo = all(
        np.array_equal(solo_out[i].round_polys, rp[rows[i]:rows[i + 1]]) and
        np.array_equal(solo_out[i].challenges, ch[rows[i]:rows[i + 1]]) and
        np.array_equal(solo_out[i].final_value, fv[i]) for i in range(count))
    assert same_as_solo, "batched proofs differ from the one-at-a-time proofs"
    del solos

    oracle_checked = 0
    cpu_b = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        O.set_threads(os.cpu_count() or 1)
        cpu_s = 0.0
        for i in range(count):
            n = 1 << nv[i]
            pr = O.Prover(O.IP, O.MSB, 3, [O.gen_table(seeds[i][0], n), O.gen_table(seeds[i][1], n)])
            t0 = time.perf_counter()
            orp, och, ofv = O.sumcheck(pr, nv[i], O.Transcript(3, label=batch_label(i)))
            cpu_s += time.perf_counter() - t0
            ok = (np.array_equal(orp, rp[rows[i]:rows[i + 1]]) and np.array_equal(och, ch[rows[i]:rows[i + 1]])
                  and np.array_equal(ofv, fv[i]))
            assert ok, "batched proof %d differs from the oracle" % i
            oracle_checked += 1
        cpu_b = cpu_rec(count, cpu_s, "proofs/s", "the %d proofs of the cohort one after another (sumcheck "
                        "time only, table generation excluded)" % count)
    verify = run_verify_batch(E, L, ctx, b, nv, rp, fv, rows)
    alg = sum(ip_fp3_bytes_as_run(n) for n in nv)
    alg_textbook = sum(ip_fp3_bytes(n) for n in nv)
    E.launch_count_reset()
    b.prove_raw(txs(), outputs=False)
    launches = E.launch_count()
    evals = sum(2 << n for n in nv)
    del b
    return {
        "workload": "%d InnerProductProver MSB instances, num_vars uniform on 10..=22 (seed 0x%X), per-instance "
                    "seeded uniform tables and transcript labels effsc-gpu/batch/{i}, Fp3 challenges, all rounds"
                    % (count, BATCH_SEED),
        "instances": count, "total_evals": evals, "algorithmic_bytes": alg,
        "algorithmic_bytes_note": "two-pass start for instances with >= 3 multi-block rounds; the tail choice "
                                  "of the autotuner changes only where the last rounds run (bytes counted "
                                  "without the tail); one pass per round would move %d bytes" % alg_textbook,
        "batched": {"ms_per_cohort": ms_batch, "proofs_per_s": count / (ms_batch * 1e-3),
                    "evals_per_s": evals / (ms_batch * 1e-3), "hbm_gbs": alg / (ms_batch * 1e-3) / 1e9,
                    "quads_per_thread": q, "tail_len": tail, "launches_per_cohort": launches,
                    "path": "effsc_batch_prove: one kernel per step for all instances in their multi-block rounds, "
                            "one tail launch, one final-fold launch, one CUDA graph, proofs copied back every step"},
        "one_at_a_time": {"ms_per_cohort": ms_solo, "proofs_per_s": count / (ms_solo * 1e-3),
                          "path": "effsc_prove per instance (its own CUDA graph), device-resident tables"},
        "speedup_proofs_per_s": ms_solo / ms_batch,
        "cpu_baseline": cpu_b,
        "autotune": tune_rec,
        "bit_exact": {"batched_vs_one_at_a_time": count, "batched_vs_oracle": oracle_checked},
        "verify": verify,
    }


def run_verify_batch(E, L, ctx, b, nv, rp, fv, rows, reps=5):
    """The batch's proofs checked by the device batch verifier
    (effsc_verify_batch, one warp per proof, host buffers in and out) and by
    the host verifier one at a time: claimed sums from the device tables
    (effsc_stream_claim), every final claim must equal the proof's final
    value, and both verifiers must agree."""
    import ctypes
    import numpy as np
    from effsc_gpu import _lib
    count = len(nv)
    claims = np.zeros((count, 3), dtype=np.uint64)
    for i in range(count):
        ptrs = (ctypes.POINTER(ctypes.c_uint64) * 2)(
            *[ctypes.cast(b.device_table(i, t), ctypes.POINTER(ctypes.c_uint64)) for t in range(2)])
        _lib.check(L.effsc_stream_claim(ctx.h, 3, 2, ptrs, 1 << nv[i], 1, claims[i].ctypes.data_as(
            ctypes.POINTER(ctypes.c_uint64))))
    polys = [np.ascontiguousarray(rp[rows[i]:rows[i + 1]]) for i in range(count)]
    labels = [batch_label(i) for i in range(count)]
    E.sumcheck_verify_batch(claims, 2, polys, [E.Transcript.keccak(3, l) for l in labels], ctx=ctx)
    t_dev = []
    for _ in range(reps):
        txs = [E.Transcript.keccak(3, l) for l in labels]
        t0 = time.perf_counter()
        fin, _ = E.sumcheck_verify_batch(claims, 2, polys, txs, ctx=ctx)
        t_dev.append(time.perf_counter() - t0)
    t_host = []
    for _ in range(max(1, reps // 2)):
        txs = [E.Transcript.keccak(3, l) for l in labels]
        t0 = time.perf_counter()
        host = [E.sumcheck_verify(claims[i], 2, nv[i], txs[i], polys[i])[1] for i in range(count)]
        t_host.append(time.perf_counter() - t0)
    accepted = sum(int(np.array_equal(fin[i], fv[i])) for i in range(count))
    agree = all(np.array_equal(fin[i], host[i]) for i in range(count))
    assert accepted == count and agree, "batch proofs rejected by a verifier"
    dev_s, host_s = float(np.median(t_dev)), float(np.median(t_host))
    return {"proofs": count, "accepted": accepted, "device_and_host_verifiers_agree": agree,
            "device_ms": dev_s * 1e3, "device_proofs_per_s": count / dev_s,
            "host_ms": host_s * 1e3, "host_proofs_per_s": count / host_s,
            "path": "effsc_verify_batch (one launch, one warp per proof; host buffers, copies and one "
                    "synchronize inside the wall-clock time) vs effsc_verify per proof on one host core"}


# ---------------------------------------------------------------------------
# the other single-proof workloads: Multilinear n=20 (Fp) and the degree-3
# Coefficient / EqFactored pair at n=24 (16 partial rounds, 32-byte hook)
# ---------------------------------------------------------------------------
def gl_mul_vec(a, b):
    """Elementwise Goldilocks product of two canonical uint64 arrays (input
    preparation only): 32-bit limb products, then 2^64 = 2^32 - 1 and
    2^96 = -1 (mod p)."""
    import numpy as np
    u = np.uint64
    M = u(0xFFFFFFFF)
    EPS = u(0xFFFFFFFF)
    P = u(0xFFFFFFFF00000001)
    a0, a1, b0, b1 = a & M, a >> u(32), b & M, b >> u(32)
    p00, p01, p10, p11 = a0 * b0, a0 * b1, a1 * b0, a1 * b1
    mid = p01 + p10
    c_mid = (mid < p01).astype(np.uint64)
    lo = p00 + (mid << u(32))
    c_lo = (lo < p00).astype(np.uint64)
    hi = p11 + (mid >> u(32)) + (c_mid << u(32)) + c_lo
    h0, h1 = hi & M, hi >> u(32)
    t0 = lo - h1
    t0 = t0 - EPS * (lo < h1).astype(np.uint64)
    r = t0 + h0 * EPS
    r = r + EPS * (r < t0).astype(np.uint64)
    return np.where(r >= P, r - P, r)


def profile_bytes(E, L, fn):
    """Algorithmic bytes of every kernel one call of fn launches (profiled,
    outside any graph)."""
    from effsc_gpu import _lib
    L.effsc_profile_clear()
    L.effsc_profile_enable(1)
    fn()
    L.effsc_profile_enable(0)
    tot, ms = 0, 0.0
    for i in range(L.effsc_profile_count()):
        name = _lib.ctypes.create_string_buffer(64)
        msv = _lib.ctypes.c_double()
        by = _lib.ctypes.c_uint64()
        _lib.check(L.effsc_profile_get(i, name, 64, _lib.ctypes.byref(msv), _lib.ctypes.byref(by)))
        tot += by.value
        ms += msv.value
    L.effsc_profile_clear()
    return tot, ms


def time_proofs(torch, stream, fn, steps):
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        out = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, out


def cpu_rec(work, seconds, unit, sample, scale=1.0):
    """A cpu_baseline record: the oracle (C restatement of the reference
    algorithms, all host threads) timed on this host."""
    return {"value": work / seconds * scale, "unit": unit, "cores": os.cpu_count() or 1, "kind": "port",
            "seconds": seconds, "sample": sample + "; C restatement of the reference algorithms (oracle/), "
                                                    "not the Rust reference binary",
            "cpu_model": cpu_model()}


def cpu_model():
    """The host CPU's model name: /proc/cpuinfo's model name (x86), else
    lscpu's (Arm: e.g. Neoverse-V2), else the Arm part number."""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        import subprocess
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        parts = {"0xd4f": "Neoverse-V2", "0xd40": "Neoverse-V1", "0xd0c": "Neoverse-N1", "0xd49": "Neoverse-N2"}
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("cpu part"):
                v = line.split(":", 1)[1].strip().lower()
                return "Arm " + parts.get(v, "part " + v)
    except OSError:
        pass
    import platform
    return platform.machine()


def run_configs(args, E, L, ctx, stream, rank):
    import numpy as np
    import torch
    res = {}
    check = rank == 0 and not args.no_cpu_baseline
    if check:
        from oracle import oracle as O
        O.set_threads(os.cpu_count() or 1)
    res["multilinear_fp_n20"] = run_ml_n20(E, L, ctx, stream, check)
    # Coefficient (eq * f * g, degree 3) and EqFactored (p = f . g), num_vars = 24
    n, rounds = 24, 16
    hook = bytes(range(32))
    w = E.gen_uniform(E.table_seed(0x3C03_2026, 0), 3 * n, ctx=ctx).reshape(n, 3)
    f = E.gen_uniform(E.table_seed(0x3C03_2026, 1), 1 << n, ctx=ctx)
    g = E.gen_uniform(E.table_seed(0x3C03_2026, 2), 1 << n, ctx=ctx)
    eq = E.build_eq_table(w, ctx=ctx)
    coef = E.CoefficientProver([eq, f, g], ctx=ctx)
    lab_c = b"effsc-gpu/coef3/v1"

    def coef_proof(use_graph=True):
        coef.reset()
        return coef.prove(rounds, E.Transcript.keccak(E.FP3, lab_c), hook=hook, use_graph=use_graph)

    ms_c, pf_c = time_proofs(torch, stream, coef_proof, 20)
    by_c, _ = profile_bytes(E, L, lambda: coef_proof(False))
    pvals = gl_mul_vec(f, g)
    eqf = E.EqFactoredProver(w, pvals, ctx=ctx)
    lab_e = b"effsc-gpu/eqf/v1"

    def eqf_proof(use_graph=True):
        eqf.reset()
        return eqf.prove(rounds, E.Transcript.keccak(E.FP3, lab_e), hook=hook, use_graph=use_graph)

    ms_e, pf_e = time_proofs(torch, stream, eqf_proof, 20)
    by_e, _ = profile_bytes(E, L, lambda: eqf_proof(False))
    ok_c = ok_e = cpu_c = cpu_e = None
    if check:
        pr = O.Prover(O.COEF, O.MSB, 3, [eq, f, g])
        t0 = time.perf_counter()
        rp, ch, fv = O.sumcheck(pr, rounds, O.Transcript(3, label=lab_c), hook=hook)
        cpu_c = cpu_rec(3 * (1 << n), time.perf_counter() - t0, "evals/s",
                        "one full proof of the same workload (same inputs, transcript and hook)")
        ok_c = bool(np.array_equal(pf_c.round_polys, rp) and np.array_equal(pf_c.final_value, fv))
        assert ok_c, "Coefficient n=24 proof differs from the oracle"
        pr = O.Prover.eq_factored(3, w, pvals)
        t0 = time.perf_counter()
        rp, ch, fv = O.sumcheck(pr, rounds, O.Transcript(3, label=lab_e), hook=hook)
        cpu_e = cpu_rec(1 << n, time.perf_counter() - t0, "evals/s",
                        "one full proof of the same workload (same inputs, transcript and hook)")
        ok_e = bool(np.array_equal(pf_e.round_polys, rp) and np.array_equal(pf_e.final_value, fv))
        assert ok_e, "EqFactored n=24 proof differs from the oracle"
    res["coefficient_eqfg_n24"] = {
        "workload": "CoefficientProver MSB with the degree-3 product evaluator on [eq(r, .) (Fp3), f, g (Fp)], "
                    "num_vars=24, r seeded uniform Fp3, 16 partial rounds + finalize, hook absorbs 0x00..0x1f per "
                    "round, label %s" % lab_c.decode(),
        "ms_per_proof": ms_c, "evals_per_s": 3 * (1 << n) / (ms_c * 1e-3), "algorithmic_bytes": by_c,
        "hbm_gbs": by_c / (ms_c * 1e-3) / 1e9, "bit_exact_vs_oracle": ok_c, "cpu_baseline": cpu_c}
    res["eq_factored_n24"] = {
        "workload": "EqFactoredProver, w = the same r, p = f . g (one base table), num_vars=24, 16 partial "
                    "rounds + finalize, same hook, label %s" % lab_e.decode(),
        "ms_per_proof": ms_e, "evals_per_s": (1 << n) / (ms_e * 1e-3), "algorithmic_bytes": by_e,
        "hbm_gbs": by_e / (ms_e * 1e-3) / 1e9, "bit_exact_vs_oracle": ok_e, "cpu_baseline": cpu_e}
    del coef, eqf
    res["gkr_k12"] = run_gkr_k12(E, L, ctx, stream, check)
    # InnerProduct LSB (pair-split), num_vars = 26: the other variant of the
    # headline configuration
    n = 26
    al = E.gen_uniform(E.table_seed(SEED, 0), 1 << n, ctx=ctx)
    bl = E.gen_uniform(E.table_seed(SEED, 1), 1 << n, ctx=ctx)
    lsb = E.InnerProductProverLSB(al, bl, field=E.FP3, ctx=ctx)
    lab_l = b"effsc-gpu/ip-lsb/v1"

    def lsb_proof(use_graph=True):
        lsb.reset()
        return lsb.prove(n, E.Transcript.keccak(E.FP3, lab_l), use_graph=use_graph)

    ms_l, pf_l = time_proofs(torch, stream, lsb_proof, 10)
    by_l, _ = profile_bytes(E, L, lambda: lsb_proof(False))
    ok_l = cpu_l = None
    if check:
        pr = O.Prover(O.IP, O.LSB, 3, [al, bl])
        t0 = time.perf_counter()
        rp, ch, fv = O.sumcheck(pr, n, O.Transcript(3, label=lab_l))
        cpu_l = cpu_rec(2 * (1 << n), time.perf_counter() - t0, "evals/s", "one full proof of the same workload")
        ok_l = bool(np.array_equal(pf_l.round_polys, rp) and np.array_equal(pf_l.final_value, fv))
        assert ok_l, "InnerProduct LSB n=26 proof differs from the oracle"
    res["inner_product_lsb_n26"] = {
        "workload": "InnerProductProverLSB (pairs 2k, 2k+1), num_vars=26, a, b = the headline's seeded tables, Fp3 "
                    "challenges, 26 rounds + finalize, label %s" % lab_l.decode(),
        "ms_per_proof": ms_l, "evals_per_s": 2 * (1 << n) / (ms_l * 1e-3), "algorithmic_bytes": by_l,
        "hbm_gbs": by_l / (ms_l * 1e-3) / 1e9, "bit_exact_vs_oracle": ok_l, "cpu_baseline": cpu_l}
    del lsb, al, bl
    # InnerProduct n = 28 over tables left in host memory and read in place
    # (the path for tables larger than HBM): only the Fp3 tables of length
    # N/4 are allocated on the device
    n = 28
    ah = E.gen_uniform(E.table_seed(0x4057_2026, 0), 1 << n, ctx=ctx)
    bh = E.gen_uniform(E.table_seed(0x4057_2026, 1), 1 << n, ctx=ctx)
    hp = E.InnerProductProver.from_host([ah, bh], field=E.FP3, ctx=ctx)
    lab_h = b"effsc-gpu/host/v1"

    def host_proof(use_graph=True):
        hp.reset()
        return hp.prove(n, E.Transcript.keccak(E.FP3, lab_h), use_graph=use_graph)

    ms_h, pf_h = time_proofs(torch, stream, host_proof, 5)
    ok_h = cpu_h = None
    if check:
        pr = O.Prover(O.IP, O.MSB, 3, [ah, bh])
        t0 = time.perf_counter()
        rp, ch, fv = O.sumcheck(pr, n, O.Transcript(3, label=lab_h))
        cpu_h = cpu_rec(2 * (1 << n), time.perf_counter() - t0, "evals/s", "one full proof of the same workload")
        ok_h = bool(np.array_equal(pf_h.round_polys, rp) and np.array_equal(pf_h.final_value, fv))
        assert ok_h, "host-resident InnerProduct proof differs from the oracle"
    N = 1 << n
    res["inner_product_host_tables_n28"] = {
        "workload": "InnerProductProver MSB, num_vars=28, a, b = 2^28 seeded uniform values each in pageable host "
                    "memory (2 x 2 GiB), read in place by the GPU through host page tables; Fp3 challenges, all rounds, "
                    "label %s" % lab_h.decode(),
        "ms_per_proof": ms_h, "evals_per_s": 2 * N / (ms_h * 1e-3),
        "host_bytes_read_per_proof": 2 * 16 * N,
        "host_read_gbs": 2 * 16 * N / (ms_h * 1e-3) / 1e9,
        "device_table_bytes": 2 * 3 * (N // 4) * 8,
        "device_table_bytes_if_uploaded": 2 * N * 8 + 2 * 3 * (N // 4) * 8,
        "bit_exact_vs_oracle": ok_h, "cpu_baseline": cpu_h}
    del hp, ah, bh
    res["protogalaxy_fold"] = run_pg_fold(E, L, ctx, stream, check)
    return res


def run_ml_n20(E, L, ctx, stream, check, steps=200):
    """Multilinear MSB over Fp, num_vars = 20 (config 1), all rounds."""
    import numpy as np
    import torch
    if check:
        from oracle import oracle as O
    n = 20
    v = E.gen_uniform(E.table_seed(0x3170_2026, 0), 1 << n, ctx=ctx)
    ml = E.MultilinearProver(v, field=E.FP, ctx=ctx)
    lab = b"effsc-gpu/ml/v1"

    def ml_proof(use_graph=True):
        ml.reset()
        return ml.prove(n, E.Transcript.keccak(E.FP, lab), use_graph=use_graph)

    ms, pf = time_proofs(torch, stream, ml_proof, steps)
    by, _ = profile_bytes(E, L, lambda: ml_proof(False))
    ok = cpu = None
    if check:
        pr = O.Prover(O.ML, O.MSB, 1, [v])
        t0 = time.perf_counter()
        rp, ch, fv = O.sumcheck(pr, n, O.Transcript(1, label=lab))
        cpu = cpu_rec(1 << n, time.perf_counter() - t0, "evals/s", "one full proof of the same workload")
        ok = bool(np.array_equal(pf.round_polys.reshape(n, 1), rp[:, :, 0]) and
                  np.array_equal(pf.final_value.reshape(1), fv[:1]))
        assert ok, "Multilinear n=20 proof differs from the oracle"
    return {
        "workload": "MultilinearProver MSB over Fp, num_vars=20, seeded uniform table, Fp challenges, label %s, "
                    "20 rounds + finalize; one CUDA graph per proof (L2-resident, latency-bound)" % lab.decode(),
        "us_per_proof": ms * 1e3, "evals_per_s": (1 << n) / (ms * 1e-3), "algorithmic_bytes": by,
        "hbm_gbs": by / (ms * 1e-3) / 1e9, "bit_exact_vs_oracle": ok, "cpu_baseline": cpu}


def run_gkr_k12(E, L, ctx, stream, check, steps=20):
    """GkrProver, k = 12: add, mult of 2^24 base entries, w of 2^12, 24 rounds."""
    import numpy as np
    import torch
    if check:
        from oracle import oracle as O
    k = 12
    add = E.gen_uniform(E.table_seed(0x6C12_2026, 0), 1 << (2 * k), ctx=ctx)
    mult = E.gen_uniform(E.table_seed(0x6C12_2026, 1), 1 << (2 * k), ctx=ctx)
    wv = E.gen_uniform(E.table_seed(0x6C12_2026, 2), 1 << k, ctx=ctx)
    gk = E.GkrProver(add, mult, wv, ctx=ctx)
    lab_g = b"effsc-gpu/gkr/v1"

    def gkr_proof(use_graph=True):
        gk.reset()
        return gk.prove(2 * k, E.Transcript.keccak(E.FP3, lab_g), use_graph=use_graph)

    ms_g, pf_g = time_proofs(torch, stream, gkr_proof, steps)
    by_g, _ = profile_bytes(E, L, lambda: gkr_proof(False))
    ok_g = cpu_g = None
    if check:
        orc = O.Prover.gkr(3, add, mult, wv)
        t0 = time.perf_counter()
        rp, ch, fv = O.sumcheck(orc, 2 * k, O.Transcript(3, label=lab_g))
        cpu_g = cpu_rec(2 * (1 << (2 * k)), time.perf_counter() - t0, "evals/s", "one full proof of the same workload")
        ok_g = bool(np.array_equal(pf_g.round_polys, rp) and np.array_equal(pf_g.final_value, fv)
                    and np.array_equal(gk.claimed_w_values(), orc.claimed_w_values()))
        assert ok_g, "GkrProver k=12 proof differs from the oracle"
    return {
        "workload": "GkrProver (MSB), k=12: add, mult seeded uniform tables of 2^24 Goldilocks values, w of 2^12, "
                    "Fp3 challenges, 24 rounds + finalize, label %s; witness kept as two 2^12 tables" % lab_g.decode(),
        "ms_per_proof": ms_g, "evals_per_s": 2 * (1 << (2 * k)) / (ms_g * 1e-3), "algorithmic_bytes": by_g,
        "hbm_gbs": by_g / (ms_g * 1e-3) / 1e9, "bit_exact_vs_oracle": ok_g, "cpu_baseline": cpu_g}


def run_pg_fold(E, L, ctx, stream, check, steps=20):
    """protogalaxy::fold (effsc_protogalaxy_fold) on 2^22 polynomials of
    degree 7 over Fp (256 MiB) and 2^20 over Fp3 (192 MiB), all levels,
    coefficients resident in HBM (generated on the device); the call's own
    time (pairs upload, the passes, result read-back) by CUDA events, and the
    oracle on the same input for parity and the CPU time."""
    import numpy as np
    import torch
    from effsc_gpu import _lib
    out = {}
    for field, logn in ((1, 22), (3, 20)):
        n, width = 1 << logn, 8
        words = n * width * field
        buf = torch.empty(words, dtype=torch.int64, device="cuda")
        _lib.check(L.effsc_gen_uniform(ctx.h, E.table_seed(0x9A1F_2026, field), words,
                                       _lib.ctypes.cast(_lib.ctypes.c_void_p(buf.data_ptr()), _lib.u64p), None))
        pairs = [tuple(E.gen_uniform(E.table_seed(0x9A1F_2026, 100 + 2 * k + h), field, ctx=ctx) for h in range(2))
                 for k in range(logn)]

        def fold():
            return E.protogalaxy_fold_raw(pairs, buf.data_ptr(), n, width, field=field, ctx=ctx)

        for _ in range(3):
            got = fold()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(steps):
            got = fold()
        e1.record(stream)
        torch.cuda.synchronize()
        wall_ms = (time.perf_counter() - t0) * 1e3 / steps
        ms = e0.elapsed_time(e1) / steps
        E.launch_count_reset()
        fold()
        launches = E.launch_count()
        in_bytes = words * 8
        ok, cpu_s = None, None
        if check:
            from oracle import oracle as O
            host = buf.cpu().numpy().view(np.uint64).reshape((n, width) if field == 1 else (n, width, 3))
            t0 = time.perf_counter()
            want = O.protogalaxy_fold(pairs, host)
            cpu_s = time.perf_counter() - t0
            ok = bool(np.array_equal(np.asarray(got).reshape(-1, field), want[:, :field]) and not want[:, field:].any())
            assert ok, "protogalaxy fold differs from the oracle"
        out["%s_n2^%d_deg%d" % ("fp" if field == 1 else "fp3", logn, width - 1)] = {
            "workload": "protogalaxy::fold of 2^%d seeded uniform %s polynomials of degree %d (AoS, %d MiB), %d levels "
                        "with seeded (a, b), result of degree %d" % (logn, "Fp" if field == 1 else "Fp3", width - 1,
                                                                     in_bytes >> 20, logn, width - 1 + logn),
            "ms_per_fold": ms, "wall_ms_per_fold": wall_ms, "coefficients_per_s": n * width / (ms * 1e-3),
            "input_bytes": in_bytes, "hbm_gbs": in_bytes / (ms * 1e-3) / 1e9, "launches_per_fold": launches,
            "cpu_oracle_s": cpu_s, "cpu_cores": os.cpu_count(), "bit_exact_vs_oracle": ok,
            "cpu_baseline": cpu_rec(n * width, cpu_s, "coefficients/s", "one fold of the same input")
            if cpu_s else None}
        del buf
    return out


# ---------------------------------------------------------------------------
# serving: open-loop Poisson stream under an HBM budget
# ---------------------------------------------------------------------------
SERVE_SEED = 0x5E7E_2026


def serve_workload(count):
    """70% InnerProduct / 30% Multilinear, num_vars uniform on the integers
    14..=26 (table size log-uniform), per-request seeds; all seeded."""
    import random
    rng = random.Random(SERVE_SEED)
    kinds, nv = [], []
    for _ in range(count):
        kinds.append(1 if rng.random() < 0.7 else 0)
        nv.append(rng.randint(14, 26))
    return kinds, nv


def serve_label(i):
    return ("effsc-gpu/serve/%d" % i).encode()


def run_serving(args, E, ctx):
    import numpy as np
    count = args.serve_requests
    kinds, nv = serve_workload(count)
    seeds = np.array([[E.table_seed(SERVE_SEED + i, t) for t in range(2)] for i in range(count)], dtype=np.uint64)
    srv = E.Server(hbm_budget=int(args.serve_budget_gb * 1e9), max_active=args.serve_slots, ctx=ctx)

    def trace(arrivals, sub=None, proofs=False):
        idx = range(count) if sub is None else sub
        txs = [E.Transcript.keccak(E.FP3, serve_label(i)) for i in idx]
        return srv.run_trace([kinds[i] for i in idx], [nv[i] for i in idx], seeds[list(idx)], txs,
                             arrivals, proofs=proofs)

    # warm-up: fills the server's memory pool up to the budget's working set
    warm = list(range(min(count, 400)))
    trace(np.zeros(len(warm)), sub=warm)
    # saturation: every request offered at t = 0
    lat_sat, mk_sat, proofs_sat = trace(np.zeros(count), proofs=True)
    sat = count / mk_sat
    rng = np.random.default_rng(SERVE_SEED)
    levels = {}
    proofs_full = None
    for frac in (0.5, 0.8, 1.0):
        rate = frac * sat
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=count))
        lat, mk, pr = trace(arrivals, proofs=frac == 1.0)
        if pr is not None:
            proofs_full = pr
        levels["%d%%" % int(frac * 100)] = {
            "offered_proofs_per_s": rate, "sustained_proofs_per_s": count / mk,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "makespan_s": mk}
    # the same request gives the same proof in both mixes, and alone
    same_mix = all(np.array_equal(proofs_sat[i].round_polys, proofs_full[i].round_polys)
                   and np.array_equal(proofs_sat[i].final_value, proofs_full[i].final_value) for i in range(count))
    assert same_mix, "a serving proof depends on the mix"
    sample = sorted(set([int(i) for i in np.linspace(0, count - 1, 12)]) | {int(np.argmax(nv)), int(np.argmin(nv))})
    for i in sample:
        n = nv[i]
        tabs = [E.gen_uniform(int(seeds[i][t]), 1 << n, ctx=ctx) for t in range(2 if kinds[i] == 1 else 1)]
        p = (E.InnerProductProver(tabs[0], tabs[1], ctx=ctx) if kinds[i] == 1 else E.MultilinearProver(tabs[0], ctx=ctx))
        ref = p.prove(n, E.Transcript.keccak(E.FP3, serve_label(i)))
        assert np.array_equal(ref.round_polys, proofs_full[i].round_polys) and \
            np.array_equal(ref.final_value, proofs_full[i].final_value), "serving proof %d differs from alone" % i
        del p, tabs
    host_fed = serving_host_leg(args, E, ctx, srv, kinds, nv) if args.serve_host_requests else None
    del srv
    # CPU baseline: the oracle proves the same sample of the mix one request
    # after another (bounded: the sample, not all requests)
    cpu_s = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.set_threads(os.cpu_count() or 1)
        cpu_s = 0.0
        for i in sample:
            n = 1 << nv[i]
            tabs = [O.gen_table(int(seeds[i][t]), n) for t in range(2 if kinds[i] == 1 else 1)]
            pr = O.Prover(O.IP if kinds[i] == 1 else O.ML, O.MSB, 3, tabs)
            t0 = time.perf_counter()
            rp, _, fv = O.sumcheck(pr, nv[i], O.Transcript(3, label=serve_label(i)))
            cpu_s += time.perf_counter() - t0
            assert np.array_equal(rp[:, :rp.shape[1] if kinds[i] == 1 else 1],
                                  np.asarray(proofs_full[i].round_polys).reshape(nv[i], -1, 3)), \
                "serving proof %d differs from the oracle" % i
    mean_nv_sample = sum(nv[i] for i in sample) / len(sample)
    return {
        "workload": "%d requests, 70%% InnerProductProver / 30%% MultilinearProver (MSB), num_vars uniform on "
                    "14..=26 (seed 0x%X), uniform Goldilocks tables generated on the device per request, Fp3 "
                    "challenges, labels effsc-gpu/serve/{i}; open-loop Poisson arrivals" % (count, SERVE_SEED),
        "hbm_budget_gb": args.serve_budget_gb, "slots": args.serve_slots,
        "saturation": {"proofs_per_s": sat, "p50_ms": float(np.percentile(lat_sat, 50) * 1e3),
                       "p99_ms": float(np.percentile(lat_sat, 99) * 1e3), "makespan_s": mk_sat},
        "rates": levels,
        "host_fed": host_fed,
        "latency": "submission (arrival) to the proof in host memory",
        "bit_exact": {"same_in_both_mixes": count, "equal_to_alone_sample": len(sample),
                      "equal_to_oracle_sample": len(sample) if cpu_s is not None else 0},
        "cpu_baseline": cpu_rec(len(sample), cpu_s, "proofs/s",
                                "%d requests of the mix (evenly spaced indices plus the largest and smallest, "
                                "mean num_vars %.1f) proved one after another" % (len(sample), mean_nv_sample))
        if cpu_s else None,
    }


def serving_host_leg(args, E, ctx, srv, kinds, nv):
    """The serving mix with every request's tables in pinned host memory: the
    upload over the host link is part of each request's latency.  One pinned
    table pair per num_vars (2 x 8 x 2^n bytes, about 2 GiB for 14..26) is
    shared by the requests of that size; each request keeps its own
    transcript label.  Saturation, then Poisson arrivals at 50/80/100% of the
    host-fed saturation rate; every proof equal across the two mixes and a
    sample equal to the same request proved alone."""
    import numpy as np
    import torch
    count = min(args.serve_host_requests, len(kinds))
    sizes = sorted(set(nv[:count]))
    pinned, host_np = {}, {}
    for n in sizes:
        arrs = [E.gen_uniform(E.table_seed(SERVE_SEED ^ 0x4057, 64 * n + t), 1 << n, ctx=ctx) for t in range(2)]
        host_np[n] = arrs
        pinned[n] = [torch.from_numpy(a.view(np.int64)).pin_memory() for a in arrs]
    host = [[pinned[nv[i]][t].data_ptr() for t in range(2 if kinds[i] == 1 else 1)] for i in range(count)]
    upload_bytes = sum(8 * (1 << nv[i]) * (2 if kinds[i] == 1 else 1) for i in range(count))

    def trace(arrivals, proofs=False):
        txs = [E.Transcript.keccak(E.FP3, serve_label(i)) for i in range(count)]
        return srv.run_trace(kinds[:count], nv[:count], None, txs, arrivals, proofs=proofs, host_tables=host)

    trace(np.zeros(count))   # warm-up
    lat_sat, mk_sat, proofs_sat = trace(np.zeros(count), proofs=True)
    sat = count / mk_sat
    rng = np.random.default_rng(SERVE_SEED + 1)
    levels = {}
    proofs_full = None
    for frac in (0.5, 0.8, 1.0):
        rate = frac * sat
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=count))
        lat, mk, pr = trace(arrivals, proofs=frac == 1.0)
        if pr is not None:
            proofs_full = pr
        levels["%d%%" % int(frac * 100)] = {
            "offered_proofs_per_s": rate, "sustained_proofs_per_s": count / mk,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "makespan_s": mk}
    same_mix = all(np.array_equal(proofs_sat[i].round_polys, proofs_full[i].round_polys)
                   and np.array_equal(proofs_sat[i].final_value, proofs_full[i].final_value) for i in range(count))
    assert same_mix, "a host-fed serving proof depends on the mix"
    sample = sorted(set([int(i) for i in np.linspace(0, count - 1, 10)]) |
                    {int(np.argmax(nv[:count])), int(np.argmin(nv[:count]))})
    for i in sample:
        n = nv[i]
        t = host_np[n]
        p = (E.InnerProductProver(t[0], t[1], ctx=ctx) if kinds[i] == 1 else E.MultilinearProver(t[0], ctx=ctx))
        ref = p.prove(n, E.Transcript.keccak(E.FP3, serve_label(i)))
        assert np.array_equal(ref.round_polys, proofs_full[i].round_polys) and \
            np.array_equal(ref.final_value, proofs_full[i].final_value), "host-fed proof %d differs from alone" % i
        del p
    del pinned, host_np
    return {
        "workload": "the first %d requests of the same mix (kinds, num_vars, labels), tables read from pinned host "
                    "memory (one seeded table pair per num_vars) and uploaded on admission" % count,
        "upload_bytes": upload_bytes,
        "saturation": {"proofs_per_s": sat, "p50_ms": float(np.percentile(lat_sat, 50) * 1e3),
                       "p99_ms": float(np.percentile(lat_sat, 99) * 1e3), "makespan_s": mk_sat,
                       "upload_gbs": upload_bytes / mk_sat / 1e9},
        "rates": levels,
        "bit_exact": {"same_in_both_mixes": count, "equal_to_alone_sample": len(sample)},
    }


def main():
    args = parse()
    if args.only:
        run_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


def run_plain_proofs(E, ctx, stream, which, n, steps):
    """`steps` proofs of one workload at num_vars = n, launched kernel by
    kernel (no graph), for launch lists and kernel captures: the headline's
    InnerProduct (MSB or LSB, seeded tables, Fp3 challenges) or the
    Coefficient eq * f * g workload (16 rounds, or n - 1 when n <= 16, with
    the 32-byte hook)."""
    import time
    import torch
    if which == "coefficient_eqfg":
        w = E.gen_uniform(E.table_seed(0x3C03_2026, 0), 3 * n, ctx=ctx).reshape(n, 3)
        f = E.gen_uniform(E.table_seed(0x3C03_2026, 1), 1 << n, ctx=ctx)
        g = E.gen_uniform(E.table_seed(0x3C03_2026, 2), 1 << n, ctx=ctx)
        prover = E.CoefficientProver([E.build_eq_table(w, ctx=ctx), f, g], ctx=ctx)
        rounds, hook, label = min(16, n - 1), bytes(range(32)), b"effsc-gpu/coef3/v1"
    else:
        a = E.gen_uniform(E.table_seed(SEED, 0), 1 << n, ctx=ctx)
        b = E.gen_uniform(E.table_seed(SEED, 1), 1 << n, ctx=ctx)
        cls = E.InnerProductProver if which == "inner_product_msb" else E.InnerProductProverLSB
        prover = cls(a, b, field=E.FP3, ctx=ctx)
        rounds, hook, label = n, b"", LABEL
    t0 = time.perf_counter()
    for _ in range(steps):
        prover.reset()
        pf = prover.prove(rounds, E.Transcript.keccak(E.FP3, label), hook=hook, use_graph=False)
    torch.cuda.synchronize()
    return {"workload": which, "num_vars": n, "rounds": rounds, "proofs": steps,
            "wall_ms_per_proof": (time.perf_counter() - t0) * 1e3 / steps,
            "final_value": [int(x) for x in pf.final_value.reshape(-1)]}


def run_only(args):
    import torch
    import effsc_gpu as E
    L = E.load()
    ctx = E.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    check = not args.no_cpu_baseline
    if args.only in ("inner_product_msb", "inner_product_lsb", "coefficient_eqfg"):
        rec = run_plain_proofs(E, ctx, stream, args.only, args.num_vars, max(args.steps, 1))
    elif args.only == "protogalaxy_fold":
        rec = run_pg_fold(E, L, ctx, stream, check, steps=max(args.steps, 1))
    elif args.only == "multilinear_n20":
        rec = run_ml_n20(E, L, ctx, stream, check, steps=max(args.steps, 1))
    else:
        rec = run_gkr_k12(E, L, ctx, stream, check, steps=max(args.steps, 1))
    print(json.dumps({"only": args.only, "record": rec}))


if __name__ == "__main__":
    main()
