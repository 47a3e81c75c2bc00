#!/usr/bin/env python
"""Basefold commit+open throughput on GB300.

Workload: the plain single-polynomial prover step of han0110/learn-zkp's
Basefold over POLYVAL with the binary Reed–Solomon code — commit (encode +
Keccak-256 Merkle tree), eval at a random point, open (interleaved sumcheck /
fold rounds + 309 query openings) — for 2^24 evaluations at blowup 2, one
column, lambda = 128.  Inputs are synthetic (SplitMix64, seed 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on stdout (rank 0).  `value` is commit+open per second with the
evaluations already resident in HBM; `e2e` is the same through the C ABI with
host buffers (H2D of the evaluations and D2H of the proof inside the timed
region).  Multi-GPU runs are independent replicas (the path does not shard).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "learn-zkp_gb300"))
sys.path.insert(0, ROOT)

METRIC = "Basefold commit+open/sec at 2^20-2^24, batched vs plain on GB300; p99 latency"
UNIT = "commit+open/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", type=int, default=24, help="log2 of the number of evaluations")
    ap.add_argument("--log2-c", type=int, default=1, help="log2 of the blowup")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and served workloads")
    ap.add_argument("--profile-only", action="store_true", help="warmup + steps, no JSON extras (for ncu)")
    ap.add_argument("--profile-sumcheck", type=int, nargs=2, metavar=("K", "N"),
                    help="one product sumcheck of K polys over 2^N points, nothing else (for ncu)")
    ap.add_argument("--profile-verify", type=int, nargs=2, metavar=("N", "COUNT"),
                    help="one batched verify of COUNT proofs of 2^N evaluations, nothing else (for ncu)")
    ap.add_argument("--profile-wide", type=int, metavar="LOG_N",
                    help="one commit + eval + open of a 2^LOG_N x 256 Polyval matrix (the reference's binary "
                         "bench shape), nothing else (for ncu)")
    ap.add_argument("--profile-prime", type=int, nargs=3, metavar=("GENERIC", "LOG_N", "LOG_POLYS"),
                    help="one prime-field commit + open (GENERIC 0: Reed-Solomon, 1: generic code with "
                         "log2_k_0 = 3) of a 2^LOG_N x 2^LOG_POLYS BabyBear matrix, nothing else (for ncu)")
    return ap.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        backend = "nccl" if args.impl == "gb300" else "gloo"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def throughput(ws, steps, ms):
    """Whole-job rate: every rank ran `steps` steps; `ms` is the slowest rank's time."""
    return ws * steps / (ms / 1e3)


def max_over_ranks(ws, v, device=None):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.proc = device, None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes(n, log2_c):
    """Minimal compulsory DRAM bytes of one commit+open (width 1): commit
    (16 + 80c) N, open (112c + 72) N."""
    N, c = 1 << n, 1 << log2_c
    return (16 + 80 * c) * N + (112 * c + 72) * N


def tree_nodes(n, log2_c):
    """Inner Merkle nodes hashed per commit+open: codeword tree + folded-codeword trees."""
    nd = 1 << (n + log2_c)
    return (nd - 1) + sum(((1 << log2_c) << i) - 1 for i in range(n))


# Integer-pipe instruction counts (ncu, this build): a Keccak-f[1600]
# permutation on bit-interleaved lanes is 4116 ALU-pipe instructions; a
# GF(2^128) product is 144 IMAD.WIDE (FMA pipe) plus about 276 ALU-pipe
# instructions (masks, XORs, Karatsuba sums, reduction).  The ALU pipe
# retires 64 thread-instructions per clock per SM, IMAD.WIDE 24.
KECCAK_ALU, GF_ALU, GF_IMAD_WIDE = 4116, 276, 144


def proof_work(n, log2_c):
    """(Keccak-f permutations, GF products) of one commit+eval+open, width 1:
    codeword leaves and tree, every folded-codeword tree (basefold.rs:350-355);
    encode (c n N / 2), eval (N), eq table, round reductions, fixes and folds."""
    N, c = 1 << n, 1 << log2_c
    perms = c * N + (c * N - 1) + sum(2 * (c << i) - 1 for i in range(n))
    gf = (c * n // 2 + 2 * c + 3) * N
    return perms, gf


def proof_floor_ms(n, log2_c, sm_mhz, num_sms):
    """Instruction floor of one proof: its ALU-pipe instructions at 64 per
    clock per SM, or its IMAD.WIDE at 24, whichever is longer."""
    perms, gf = proof_work(n, log2_c)
    clk = sm_mhz * 1e6 * num_sms
    alu = (perms * KECCAK_ALU + gf * GF_ALU) / (64.0 * clk)
    fma = gf * GF_IMAD_WIDE / (24.0 * clk)
    return 1e3 * max(alu, fma)


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0}, "fallback"


def load_traffic(name="level_kernel_traffic.json"):
    try:
        return json.load(open(os.path.join(ROOT, "profiles", name)))
    except OSError:
        return None


def cpu_step_oracle(n, log2_c):
    """One full commit+eval+open of the oracle (C++ restatement of the
    reference's CPU path) on all host cores; returns seconds."""
    from oracle import oracle as O
    from basefold_gpu import rand

    data = rand.random_elems((1 << n) + n, 0)
    O.set_threads(os.cpu_count() or 1)
    t = time.perf_counter()
    O.commit_eval_open(n, log2_c, data[: 1 << n], data[1 << n:])
    return time.perf_counter() - t


def run_reference(args, ws, rank):
    """The reference arm: the reference's CPU path (Rust) cannot be built here,
    so its C++ restatement (oracle) is timed on the host cores."""
    if rank != 0:
        return
    from oracle import oracle as O

    O.lib()
    # every requested step is a full commit+eval+open (about 5 s each on 16
    # Grace cores at 2^24); capped at 40 steps so a run stays within minutes
    W, K = min(args.warmup, 5), min(args.steps, 40)
    for _ in range(W):
        cpu_step_oracle(args.n, args.log2_c)
    ts = [cpu_step_oracle(args.n, args.log2_c) for _ in range(K)]
    total = sum(ts)
    value = K / total
    cores = os.cpu_count() or 1
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": K,
        "warmup": W, "ms_per_step": 1e3 * total / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "gf2^128+keccak-u64", "data": "synthetic (SplitMix64 seed 0)",
        "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"full commit+eval+open at 2^{args.n}, {K} steps (warmup {W}); C++ restatement "
                                   "of the reference CPU path (Rust toolchain absent)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def gen_inputs(sizes, seed):
    """One synthetic input per distinct size (reused by jobs of that size)."""
    from basefold_gpu import rand

    inputs = {}
    for n in sorted(set(sizes)):
        data = rand.random_elems((1 << n) + n, seed + n)
        inputs[n] = (data[: 1 << n], data[1 << n:])
    return inputs


def release(*objs):
    """Frees engines, pcs objects (and their memory pools) and device inputs
    of one phase before the next is timed."""
    import gc

    import torch

    for o in objs:
        if isinstance(o, dict):
            o.clear()
    del objs
    gc.collect()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def run_batched(bg, torch, device, log2_c, count=256, lo=10, hi=22, seed=4):
    """Config 4: `count` polynomials with sizes log-uniform in 2^lo..2^hi.
    Plain = commit/eval/open one at a time through the public API; batched =
    the engine with all jobs in flight.  Inputs device-resident in both."""
    import hashlib

    import numpy as np

    sizes = [int(x) for x in np.random.default_rng(seed).integers(lo, hi + 1, count)]
    inputs = gen_inputs(sizes, 1000)
    dev = {n: torch.from_numpy(ev).to(f"cuda:{device}") for n, (ev, _) in inputs.items()}
    pcs = {n: bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=device)
           for n in inputs}

    def plain_one(n):
        comm = pcs[n].commit_device(dev[n].data_ptr(), keep=dev[n])
        ch = bg.GenericChallenger.keccak256()
        ch.observe(comm.root)
        vals = pcs[n].eval(pcs[n].data(comm), inputs[n][1])
        ch.observe_ext_slice(vals)
        proof = pcs[n].open(comm, [bg.PolyEvals(vals, inputs[n][1])], ch)
        comm.free()
        return proof

    for n in inputs:  # warm every size
        plain_one(n)
    torch.cuda.synchronize()
    t = time.perf_counter()
    plain = [plain_one(n) for n in sizes]
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t
    eng = bg.Engine(device=device, log2_c=log2_c, max_inflight=32)
    jobs = [(n, dev[n].data_ptr(), inputs[n][1]) for n in sizes]
    eng.prove([(n, dev[n].data_ptr(), inputs[n][1]) for n in inputs], device_input=True)  # every size set up
    torch.cuda.synchronize()
    t = time.perf_counter()
    res = eng.prove(jobs, device_input=True)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t
    identical = all(r["proof"] == p for r, p in zip(res, plain))
    digest = hashlib.sha256(b"".join(hashlib.sha256(p).digest() for p in plain)).hexdigest()
    # the latency-bound share alone: the jobs of at most 2^16 evaluations
    small = [n for n in sizes if n <= 16]
    torch.cuda.synchronize()
    t = time.perf_counter()
    for n in small:
        plain_one(n)
    torch.cuda.synchronize()
    t_plain_small = time.perf_counter() - t
    t = time.perf_counter()
    eng.prove([(n, dev[n].data_ptr(), inputs[n][1]) for n in small], device_input=True)
    torch.cuda.synchronize()
    t_batch_small = time.perf_counter() - t
    release(eng)
    multi = run_multi_column(bg, torch, device, log2_c, sizes, pcs)
    release(pcs, dev)
    num_sms = bg.device_info(device)["num_sms"]
    floor_s = sum(proof_floor_ms(n, log2_c, 2070.0, num_sms) for n in sizes) / 1e3
    return {"workload": f"{count} polys, sizes log-uniform 2^{lo}..2^{hi} (seed {seed}), blowup {1 << log2_c}",
            "plain_proofs_per_s": count / t_plain, "batched_proofs_per_s": count / t_batch,
            "speedup": t_plain / t_batch, "proofs_identical": identical, "proofs_sha256": digest,
            "plain_s": t_plain, "batched_s": t_batch, "max_inflight": 32, "multi_column": multi,
            "floor_s": floor_s, "batched_over_floor": t_batch / floor_s,
            "small_jobs": {"count": len(small), "plain_s": t_plain_small, "batched_s": t_batch_small,
                           "speedup": t_plain_small / t_batch_small},
            "note": "floor = the mix's integer-pipe instructions (Keccak-f 4116 ALU, GF product 276 ALU + "
                    "144 IMAD.WIDE) at 64 ALU / 24 IMAD.WIDE per clock per SM at 2070 MHz; batched = engine "
                    "with per-stream job state machines (continuous batching)"}


def run_latency(bg, torch, device, log2_c, sizes=(10, 12, 14, 16, 18, 20, 22), reps=7):
    """Latency of one commit+eval+open per size, device-resident input:
    through the trait-shaped calls one at a time (three host round trips:
    root, evaluation, proof) and as one engine job (transcript on the device,
    one round trip for the query positions), with and without its captured
    CUDA graph.  Medians of `reps` after warm-up."""
    inputs = gen_inputs(list(sizes), 7000)
    rows = []
    engines = {g: bg.Engine(device=device, log2_c=log2_c, max_inflight=1, graphs=g) for g in (False, True)}
    for n in sizes:
        ev, pt = inputs[n]
        dev = torch.from_numpy(ev).to(f"cuda:{device}")
        pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=device)

        def plain():
            comm = pcs.commit_device(dev.data_ptr(), keep=dev)
            ch = bg.GenericChallenger.keccak256()
            ch.observe(comm.root)
            vals = pcs.eval(pcs.data(comm), pt)
            ch.observe_ext_slice(vals)
            pcs.open(comm, [bg.PolyEvals(vals, pt)], ch)
            comm.free()

        def timed(f):
            for _ in range(3):
                f()
            ts = []
            for _ in range(reps):
                torch.cuda.synchronize()
                t = time.perf_counter()
                f()
                ts.append(1e3 * (time.perf_counter() - t))
            return sorted(ts)[len(ts) // 2]

        row = [n, round(timed(plain), 3)]
        for g in (False, True):
            eng = engines[g]
            row.append(round(timed(lambda: eng.prove([(n, dev.data_ptr(), pt)], device_input=True)), 3))
        rows.append(row)
        del pcs, dev
    release(engines)
    return {"cols": ["num_vars", "plain_ms", "engine_ms", "engine_graph_ms"], "rows": rows}


def run_autotune(bg, torch, device, log2_c, sizes=(20, 22, 24), reps=2):
    """The launch-shape autotuner per size: whole-step time with the default
    shapes and with the shapes bf_pcs_autotune picks (its own report), and
    the proof unchanged."""
    rows = []
    for n in sizes:
        data = bg.rand.random_elems((1 << n) + n, 8000 + n)
        ev, pt = data[: 1 << n], data[1 << n:]
        dev = torch.from_numpy(ev).to(f"cuda:{device}")
        pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=device)

        def step():
            comm = pcs.commit_device(dev.data_ptr(), keep=dev)
            ch = bg.GenericChallenger.keccak256()
            ch.observe(comm.root)
            vals = pcs.eval(pcs.data(comm), pt)
            ch.observe_ext_slice(vals)
            proof = pcs.open(comm, [bg.PolyEvals(vals, pt)], ch)
            comm.free()
            return proof

        def timed():
            step()
            torch.cuda.synchronize()
            t = time.perf_counter()
            for _ in range(5):
                step()
            torch.cuda.synchronize()
            return 1e3 * (time.perf_counter() - t) / 5

        before = step()
        default_ms = timed()
        rep = pcs.autotune(reps)
        tuned_ms = timed()
        assert step() == before, "tuned shapes changed the proof"
        rows.append([n, round(default_ms, 3), round(tuned_ms, 3), [rep["tune"][k] for k in bg.Basefold.TUNE_KEYS]])
        del pcs, dev
    bg.tune_cache_clear()
    return {"cols": ["num_vars", "default_ms", "tuned_ms", "tune"], "tune_keys": bg.Basefold.TUNE_KEYS, "rows": rows}


def run_served(bg, device, log2_c, lo=12, hi=24, per_size=10, loads=(0.25, 0.5, 0.9), seed=5):
    """Config 5: open-loop Poisson arrivals, sizes log-uniform 2^lo..2^hi, host
    inputs (H2D inside), at fractions of the measured capacity.  Each load
    level (and the capacity batch) is a stratified mix: every size per_size
    times in random order, so the offered work is the distribution's and not
    a sample's."""
    import numpy as np

    rng = np.random.default_rng(seed)
    inputs = gen_inputs(list(range(lo, hi + 1)), 2000)
    # serving policy: a free slot takes the smallest queued request, and
    # requests of <= 2^18 evaluations run on high-priority streams
    eng = bg.Engine(device=device, log2_c=log2_c, max_inflight=16, smallest_first=True, priority_max_vars=18)
    # every size set up once (twiddles, pools) before anything is timed
    eng.prove([(n, inputs[n][0], inputs[n][1]) for n in range(lo, hi + 1)])
    # capacity: saturated batch of the same size distribution
    mix = list(range(lo, hi + 1)) * per_size
    per_level = len(mix)
    cap_sizes = [int(x) for x in rng.permutation(mix)]
    eng.prove([(n, inputs[n][0], inputs[n][1]) for n in cap_sizes[:8]])
    t = time.perf_counter()
    eng.prove([(n, inputs[n][0], inputs[n][1]) for n in cap_sizes])
    capacity = per_level / (time.perf_counter() - t)
    out = {"workload": f"Poisson arrivals, sizes log-uniform 2^{lo}..2^{hi}, blowup {1 << log2_c}, "
                       f"{per_level} requests per load (each size {per_size} times, random order), host inputs, "
                       "smallest-first admission, high-priority streams for <= 2^18",
           "size_range": [lo, hi],
           "capacity_proofs_per_s": capacity, "levels": []}
    eng.start()
    for load in loads:
        rate = load * capacity
        sizes = [int(x) for x in rng.permutation(mix)]
        gaps = rng.exponential(1.0 / rate, per_level)
        lat, done = [], 0
        t0 = time.perf_counter()
        t_next = t0
        for k, n in enumerate(sizes):
            t_next += gaps[k]
            while time.perf_counter() < t_next:
                for _, r in eng.poll():
                    lat.append(r["latency_ms"])
                time.sleep(0.0002)
            eng.submit(n, inputs[n][0], inputs[n][1], tag=k)
        while len(lat) < per_level:
            for _, r in eng.poll():
                lat.append(r["latency_ms"])
            time.sleep(0.0005)
        elapsed = time.perf_counter() - t0
        lat.sort()
        out["levels"].append({"offered_load": load, "offered_rate_per_s": rate, "achieved_proofs_per_s":
                              per_level / elapsed, "p50_ms": lat[len(lat) // 2],
                              "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))], "max_ms": lat[-1]})
    eng.stop()
    release(eng)
    return out


def run_commit_sweep(bg, torch, device, sizes=(18, 20, 22, 24, 26), blowups=(1, 2), reps=3):
    """Encode + Merkle commit alone (the standalone encode/commit sweep):
    device-resident evaluations, commit time per size and blowup, its
    algorithmic bytes (16 + 80c) N as GB/s and its Keccak-f rate (2cN
    permutations: cN leaves, cN - 1 nodes of the codeword tree, plus the
    first folded-codeword tree of cN/2 leaves for width 1)."""
    out = []
    peaks, _ = load_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    for log2_c in blowups:
        for n in sizes:
            N, c = 1 << n, 1 << log2_c
            ev = torch.from_numpy(bg.rand.random_elems(N, 4000 + n)).to(f"cuda:{device}")
            pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=device)
            pcs.commit_device(ev.data_ptr(), keep=ev).free()
            torch.cuda.synchronize()
            t = time.perf_counter()
            for _ in range(reps):
                pcs.commit_device(ev.data_ptr(), keep=ev).free()
            torch.cuda.synchronize()
            ms = (time.perf_counter() - t) / reps * 1e3
            gbs = (16 + 80 * c) * N / (ms * 1e-3) / 1e9
            perms = (c * N) + (c * N - 1) + (c * N // 2 + c * N // 2 - 1)
            out.append({"num_vars": n, "blowup": c, "ms": ms, "algorithmic_gbs": gbs, "hbm_frac": gbs / hbm,
                        "keccak_perms_per_s": perms / (ms * 1e-3)})
            del ev, pcs
            torch.cuda.empty_cache()
    return out


def run_sumcheck(bg, torch, device, cases=((2, 20), (3, 20), (2, 24), (3, 24)), reps=3):
    """The product sumcheck prover alone (sum over the hypercube of the
    product of k multilinear polynomials), device-resident polynomials."""
    out = []
    for k, n in cases:
        polys = torch.from_numpy(bg.rand.random_elems(k << n, 5000 + 10 * k + n)).to(f"cuda:{device}")
        pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, 1, 0)), device=device)
        claim = bg.rand.random_elems(1, 77)
        pcs.prove_sumcheck_device(k, n, polys.data_ptr(), claim, bg.GenericChallenger(b"sumcheck"))
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            pcs.prove_sumcheck_device(k, n, polys.data_ptr(), claim, bg.GenericChallenger(b"sumcheck"))
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t) / reps * 1e3
        out.append({"k": k, "num_vars": n, "ms": ms, "points_per_s": (1 << n) / (ms * 1e-3),
                    "input_gbs": 16 * k * (1 << n) / (ms * 1e-3) / 1e9})
        del polys, pcs
    return out


def verify_workload(bg, device, log2_c, n, count, distinct=8):
    """`distinct` proofs of 2^n evaluations (the reference harness: commit,
    observe the root, evaluate, observe the values, open), repeated to
    `count`; jobs() gives fresh verify_batch arguments."""
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=device)
    items = []
    for j in range(min(distinct, count)):
        data = bg.rand.random_elems((1 << n) + n, 6000 + j)
        evals, point = data[: 1 << n], data[1 << n:]
        comm = pcs.commit(evals)
        ch = bg.GenericChallenger.keccak256()
        ch.observe(comm.root)
        values = pcs.eval(pcs.data(comm), point)
        ch.observe_ext_slice(values)
        proof = pcs.open(comm, [bg.PolyEvals(values, point)], ch.clone())
        items.append((comm.root, values, point, ch.state(), proof))
        comm.free()
    items = [items[j % len(items)] for j in range(count)]

    def jobs():
        return [(r, [bg.PolyEvals(v, p)], pf, bg.GenericChallenger.from_state(b)) for r, v, p, b, pf in items]

    return pcs, items, jobs


def run_verify(bg, device, log2_c, n=20, count=64, distinct=8, reps=5):
    """Batched verify: `count` proofs of 2^n evaluations (`distinct` different
    proofs, repeated) checked in one bf_verify_batch call, from host bytes to
    result codes; beside it the oracle's verifier (C++ restatement of the
    reference's CPU verify) over the same proofs on all host cores."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O

    pcs, items, jobs = verify_workload(bg, device, log2_c, n, count, distinct)

    assert pcs.verify_batch(jobs()) == [0] * count
    ts = []
    for _ in range(reps):
        js = jobs()
        t = time.perf_counter()
        res = pcs.verify_batch(js)
        ts.append(time.perf_counter() - t)
        assert res == [0] * count
    t_gpu = sorted(ts)[len(ts) // 2]
    O.lib()
    cores = os.cpu_count() or 1
    with ThreadPoolExecutor(cores) as ex:
        t = time.perf_counter()
        codes = list(ex.map(lambda it: O.verify(n, log2_c, it[0], it[2], it[1], it[3], it[4]), items))
        t_cpu = time.perf_counter() - t
    assert codes == [0] * count
    return {"workload": f"{count} proofs of 2^{n} evaluations, blowup {1 << log2_c}, host proof bytes in, "
                        "result codes out", "proof_bytes": len(items[0][4]),
            "gpu_proofs_per_s": count / t_gpu, "gpu_ms": t_gpu * 1e3,
            "cpu_baseline": {"proofs_per_s": count / t_cpu, "cores": cores, "kind": "port",
                             "sample": f"the same {count} proofs, one per host thread at a time"},
            "speedup": t_cpu / t_gpu}


def run_multi_column(bg, torch, device, log2_c, sizes, pcs, reps=3):
    """The reference's own batching of many polynomials (commit of a
    RowMajorMatrix with num_polys columns, open of all columns at one point,
    basefold.rs:112-232): the same size mix as the batched workload, one
    matrix per size, so 13 proofs (one tree and one fold chain each) instead
    of 256, with one evaluation point per size.  A different proof shape from
    the per-polynomial proofs: reported beside them, not in their place."""
    groups = {n: sizes.count(n) for n in sorted(set(sizes))}
    mats = {n: torch.from_numpy(bg.rand.random_elems(w << n, 3000 + n)).to(f"cuda:{device}")
            for n, w in groups.items()}
    pts = {n: bg.rand.random_elems(n, 3500 + n) for n in groups}

    def group(n, w, check=False):
        comm = pcs[n].commit_device(mats[n].data_ptr(), width=w, keep=mats[n])
        ch = bg.GenericChallenger.keccak256()
        ch.observe(comm.root)
        vals = pcs[n].eval(pcs[n].data(comm), pts[n])
        ch.observe_ext_slice(vals)
        proof = pcs[n].open(comm, [bg.PolyEvals(vals, pts[n])], ch.clone())
        if check:
            pcs[n].verify(comm.root, [bg.PolyEvals(vals, pts[n])], proof, ch.clone())
        comm.free()

    from concurrent.futures import ThreadPoolExecutor

    for n, w in groups.items():
        group(n, w, check=True)  # warm, and every proof verifies
    torch.cuda.synchronize()
    # the matrices are independent: four host threads prove them concurrently
    # (one pcs and stream per size), largest first
    order = sorted(groups, key=lambda n: -(groups[n] << n))
    best = float("inf")
    for _ in range(reps):
        t = time.perf_counter()
        with ThreadPoolExecutor(4) as ex:
            list(ex.map(lambda n: group(n, groups[n]), order))
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t)
    release(mats)
    return {"workload": f"the same {len(sizes)} polys as {len(groups)} matrices (one per size, columns = polys of "
                        "that size), one point per matrix, 4 host threads", "proofs": len(groups),
            "polys_per_s": len(sizes) / best,
            "seconds": best, "verified": True}


def prime_workload(bg, torch, device, generic, log_n, log_polys, log2_c=1, seed=7):
    """The reference's prime-field bench setup (poly-commit/benches/poly-commit.rs:
    27-58, 83-178): a 2^log_n x 2^log_polys matrix of uniform BabyBears, blowup
    2^log2_c, Reed-Solomon code or the generic code with log2_k_0 = 3 (its t's
    drawn from a seeded generator, as the bench draws them from its RNG); a
    uniform point of the extension field."""
    import numpy as np
    from basefold_gpu import prime

    w = 1 << log_polys
    rng = np.random.default_rng(seed + log_n)
    host = rng.integers(0, prime.P, size=w << log_n, dtype=np.uint64).astype(np.uint32)
    point = rng.integers(0, prime.P, size=(log_n, 5), dtype=np.uint64).astype(np.uint32)
    if generic:
        lk = 3
        d = log_n - lk
        ts = rng.integers(1, prime.P, size=((1 << (log2_c + lk)) * ((1 << d) - 1)), dtype=np.uint64).astype(np.uint32)
        code = prime.GenericRandomFoldableCode(128, log2_c, lk, d, ts)
    else:
        code = prime.ReedSolomonCode(128, log2_c, log_n)
    pcs = prime.BabyBearBasefold.setup(bg.BasefoldConfig(code), device=device)
    dev = torch.from_numpy(host.view(np.int32)).to(f"cuda:{device}")
    return pcs, host, dev, point, w


def prime_open(bg, pcs, comm, point):
    """bench_open's measured call: open of one point with a fresh
    GenericChallenger::keccak256() (poly-commit.rs:150-158)."""
    from basefold_gpu import prime

    vals = pcs.eval(comm, point)
    return pcs.open(comm, [prime.PrimePolyEvals(vals, point)], bg.GenericChallenger.keccak256())


def run_prime(bg, torch, device, sizes=(16, 17, 18, 19), log_polys=8, reps=3):
    """Prime-field Basefold on the GPU at the reference's own prime bench
    shapes: ms per commit (evaluations resident in HBM, and from pinned host
    memory) and per open, both codes; every proof checked by the verifier.
    CPU baseline: the oracle (C++ restatement, all host threads) at 2^16
    rows, timed beside the GPU at the same size."""
    import numpy as np
    from basefold_gpu import prime
    from oracle import oracle as O

    rows = []
    for generic in (0, 1):
        for log_n in sizes:
            pcs, host, dev, point, w = prime_workload(bg, torch, device, generic, log_n, log_polys)
            pin = torch.from_numpy(host.view(np.int32)).pin_memory()
            comm = pcs.commit_device(dev.data_ptr(), w, keep=dev)
            ch = bg.GenericChallenger.keccak256()
            ch.observe(comm.root)
            vals = pcs.eval(comm, point)
            prime.observe_ext_slice(ch, vals)
            proof = pcs.open(comm, [prime.PrimePolyEvals(vals, point)], ch.clone())
            pcs.verify(comm.root, [prime.PrimePolyEvals(vals, point)], proof, ch.clone())
            tc = to = th = float("inf")
            for _ in range(reps):
                torch.cuda.synchronize()
                t = time.perf_counter()
                c2 = pcs.commit_device(dev.data_ptr(), w, keep=dev)
                tc = min(tc, time.perf_counter() - t)
                c2.free()
                t = time.perf_counter()
                prime_open(bg, pcs, comm, point)
                to = min(to, time.perf_counter() - t)
                t = time.perf_counter()
                c3 = pcs.commit(pin.numpy())
                th = min(th, time.perf_counter() - t)
                c3.free()
            rows.append([["reed_solomon", "generic_k0_8"][generic], log_n, round(1e3 * tc, 2), round(1e3 * to, 2),
                         round(1e3 * th, 2), len(proof)])
            comm.free()
            release(dev, pin)
    # CPU: the oracle on all host threads at 2^16 x 256 (Reed-Solomon, the smallest size of the
    # reference's prime benches), against the GPU at the same size
    n_cpu = sizes[0]
    O.set_threads(os.cpu_count() or 1)
    pcs, host, dev, point, w = prime_workload(bg, torch, device, 0, n_cpu, log_polys)
    data = host.reshape(-1, w)
    t = time.perf_counter()
    root = O.bb_commit(n_cpu, 1, data)
    cpu_commit = time.perf_counter() - t
    _, vals, blob = O.bb_harness_prepare(n_cpu, 1, data, point)
    t = time.perf_counter()
    cpu_proof = O.bb_open(n_cpu, 1, data, point, vals, blob)
    cpu_open = time.perf_counter() - t - cpu_commit  # the oracle's open recommits first
    comm = pcs.commit_device(dev.data_ptr(), w, keep=dev)
    assert comm.root == root
    gpu_proof = pcs.open(comm, [prime.PrimePolyEvals(vals, point)], bg.GenericChallenger.from_state(blob))
    assert gpu_proof == cpu_proof
    tc = to = float("inf")
    for _ in range(reps):
        t = time.perf_counter()
        c2 = pcs.commit_device(dev.data_ptr(), w, keep=dev)
        tc = min(tc, time.perf_counter() - t)
        c2.free()
        t = time.perf_counter()
        prime_open(bg, pcs, comm, point)
        to = min(to, time.perf_counter() - t)
    comm.free()
    release(dev)
    return {"workload": f"the reference's prime benches: commit / open of a 2^log_n x {1 << log_polys} BabyBear "
                        "matrix, blowup 2, E = BabyBear^5; Reed-Solomon and generic (log2_k_0 = 3) codes",
            "cols": ["code", "log_n", "commit_ms", "open_ms", "commit_from_host_ms", "proof_bytes"], "rows": rows,
            "cpu_baseline": {"kind": "port", "cores": os.cpu_count() or 1,
                             "sample": f"oracle (C++ restatement, all host threads) at 2^{n_cpu} x {1 << log_polys}, "
                                       "Reed-Solomon; proof byte-identical to the GPU's",
                             "commit_ms": round(1e3 * cpu_commit, 1), "open_ms": round(1e3 * cpu_open, 1),
                             "gpu_commit_ms": round(1e3 * tc, 3), "gpu_open_ms": round(1e3 * to, 3)}}


def run_binary_wide(bg, torch, device, sizes=(16, 17, 18, 19), log_polys=8, reps=3):
    """The reference's binary benches at their own shape (poly-commit/benches/
    poly-commit.rs:60-74, 83-178: basefold_binary_reed_solomon_polyval, a
    2^log_n x 2^log_polys matrix, C = 1): ms per commit (evaluations in HBM)
    and per open with a fresh keccak256 challenger, every proof verified."""
    w = 1 << log_polys
    rows = []
    for n in sizes:
        pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, 1, n)), device=device)
        data = bg.rand.random_elems((w << n) + n, 40 + n)
        evals, point = data[: w << n], data[w << n:]
        dev = torch.from_numpy(evals).to(f"cuda:{device}")
        comm = pcs.commit_device(dev.data_ptr(), width=w, keep=dev)
        vals = pcs.eval(pcs.data(comm), point)
        ch = bg.GenericChallenger.keccak256()
        ch.observe(comm.root)
        ch.observe_ext_slice(vals)
        proof = pcs.open(comm, [bg.PolyEvals(vals, point)], ch.clone())
        pcs.verify(comm.root, [bg.PolyEvals(vals, point)], proof, ch.clone())
        tc = to = te = float("inf")
        for _ in range(reps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            c2 = pcs.commit_device(dev.data_ptr(), width=w, keep=dev)
            tc = min(tc, time.perf_counter() - t)
            c2.free()
            t = time.perf_counter()
            pcs.eval(pcs.data(comm), point)
            te = min(te, time.perf_counter() - t)
            t = time.perf_counter()
            pcs.open(comm, [bg.PolyEvals(vals, point)], bg.GenericChallenger.keccak256())
            to = min(to, time.perf_counter() - t)
        rows.append([n, round(1e3 * tc, 2), round(1e3 * te, 2), round(1e3 * to, 2)])
        comm.free()
        release(pcs, dev)
    # CPU: the oracle on all host threads at the smallest of these sizes, its proof
    # compared with the GPU's, both timed on the same matrix
    from oracle import oracle as O

    n_cpu = sizes[0]
    O.set_threads(os.cpu_count() or 1)
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, 1, n_cpu)), device=device)
    data = bg.rand.random_elems((w << n_cpu) + n_cpu, 40 + n_cpu)
    evals, point = data[: w << n_cpu], data[w << n_cpu:]
    t = time.perf_counter()
    root = O.commit(n_cpu, 1, evals, width=w)
    cpu_commit = time.perf_counter() - t
    _, values, blob = O.harness_prepare(n_cpu, 1, evals, point, width=w)
    t = time.perf_counter()
    cpu_proof = O.open_proof(n_cpu, 1, evals, point, values, blob, width=w)
    cpu_open = time.perf_counter() - t - cpu_commit  # the oracle's open recommits first
    dev = torch.from_numpy(evals).to(f"cuda:{device}")
    comm = pcs.commit_device(dev.data_ptr(), width=w, keep=dev)
    assert comm.root == root
    gpu_proof = pcs.open(comm, [bg.PolyEvals(values, point)], bg.GenericChallenger.from_state(blob))
    assert gpu_proof == cpu_proof
    comm.free()
    release(pcs, dev)
    gpu = rows[0]
    return {"workload": f"the reference's binary benches: a 2^log_n x {w} Polyval matrix, blowup 2",
            "cols": ["log_n", "commit_ms", "eval_ms", "open_ms"], "rows": rows,
            "cpu_baseline": {"kind": "port", "cores": os.cpu_count() or 1,
                             "sample": f"oracle (C++ restatement, all host threads) at 2^{n_cpu} x {w}; "
                                       "proof byte-identical to the GPU's",
                             "commit_ms": round(1e3 * cpu_commit, 1), "open_ms": round(1e3 * cpu_open, 1),
                             "gpu_commit_ms": gpu[1], "gpu_open_ms": gpu[3]}}


def served_cpu_reference(log2_c, size_range):
    """The served mix on the CPU reference path (C++ restatement, all host
    cores): one proof per size; sizes are uniform over the range, so the
    service-time distribution of the mix is these times with equal weight.
    Queueing is left out: the mix's CPU capacity is far below any GPU load."""
    lo, hi = size_range
    times = {n: 1e3 * cpu_step_oracle(n, log2_c) for n in range(lo, hi + 1)}
    t = sorted(times.values())
    mean = sum(t) / len(t)
    return {"kind": "port", "cores": os.cpu_count() or 1,
            "service_ms_by_size": {str(k): v for k, v in times.items()},
            "service_p50_ms": t[len(t) // 2], "service_p99_ms": t[min(len(t) - 1, int(0.99 * len(t)))],
            "capacity_proofs_per_s": 1e3 / mean,
            "note": "service time of one proof per size on the host cores, no queueing"}


def workload_config(args):
    return {"workload": f"plain Basefold commit+eval+open, 2^{args.n} evaluations, blowup {1 << args.log2_c}, "
                        "width 1, lambda 128, Keccak-256 Merkle",
            "num_vars": args.n, "log2_c": args.log2_c, "width": 1,
            "l2": "inputs larger than L2 (evaluations 16*2^n B, codeword+trees several GB)"}


def main():
    args = parse()
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        barrier(ws)
        return
    import numpy as np
    import torch

    import basefold_gpu as bg

    torch.cuda.set_device(local)
    if args.profile_sumcheck:
        k, ns = args.profile_sumcheck
        polys = torch.from_numpy(bg.rand.random_elems(k << ns, 5000 + 10 * k + ns)).to(f"cuda:{local}")
        sc_pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, 1, 0)), device=local)
        sc_pcs.prove_sumcheck_device(k, ns, polys.data_ptr(), bg.rand.random_elems(1, 77),
                                     bg.GenericChallenger(b"sumcheck"))
        torch.cuda.synchronize()
        return
    if args.profile_wide:
        wn, ww = args.profile_wide, 256
        wpcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, 1, wn)), device=local)
        wdata = bg.rand.random_elems((ww << wn) + wn, 40 + wn)
        wdev = torch.from_numpy(wdata[: ww << wn]).to(f"cuda:{local}")
        wcomm = wpcs.commit_device(wdev.data_ptr(), width=ww, keep=wdev)
        wvals = wpcs.eval(wpcs.data(wcomm), wdata[ww << wn:])
        wpcs.open(wcomm, [bg.PolyEvals(wvals, wdata[ww << wn:])], bg.GenericChallenger.keccak256())
        torch.cuda.synchronize()
        return
    if args.profile_prime:
        generic, pn, plog = args.profile_prime
        ppcs, _, pdev, ppoint, pw = prime_workload(bg, torch, local, generic, pn, plog)
        pcomm = ppcs.commit_device(pdev.data_ptr(), pw, keep=pdev)
        prime_open(bg, ppcs, pcomm, ppoint)
        torch.cuda.synchronize()
        return
    if args.profile_verify:
        vn, vcount = args.profile_verify
        vpcs, _, vjobs = verify_workload(bg, local, args.log2_c, vn, vcount)
        assert vpcs.verify_batch(vjobs()) == [0] * vcount
        return
    stream = torch.cuda.current_stream()
    n, log2_c = args.n, args.log2_c
    pcs = bg.Basefold.setup(bg.BasefoldConfig(bg.BinaryReedSolomonCode(128, log2_c, n)), device=local,
                            stream=stream.cuda_stream)
    data = bg.rand.random_elems((1 << n) + n, seed=rank)
    evals, point = data[: 1 << n], data[1 << n:]
    dev = torch.from_numpy(evals).to(f"cuda:{local}")
    host = torch.from_numpy(evals).pin_memory()

    def step_device():
        comm = pcs.commit_device(dev.data_ptr(), keep=dev)
        ch = bg.GenericChallenger.keccak256()
        ch.observe(comm.root)
        vals = pcs.eval(pcs.data(comm), point)
        ch.observe_ext_slice(vals)
        proof = pcs.open(comm, [bg.PolyEvals(vals, point)], ch)
        comm.free()
        return proof

    def step_host():
        comm = pcs.commit(host.numpy())  # H2D of the pinned evaluations inside bf_commit
        ch = bg.GenericChallenger.keccak256()
        ch.observe(comm.root)
        vals = pcs.eval(pcs.data(comm), point)
        ch.observe_ext_slice(vals)
        proof = pcs.open(comm, [bg.PolyEvals(vals, point)], ch)  # D2H of the proof inside bf_open
        comm.free()
        return proof

    for _ in range(args.warmup):
        proof = step_device()
    if args.profile_only:
        for _ in range(args.steps):
            step_device()
        torch.cuda.synchronize()
        return

    # ---- timed region: device-resident inputs ----------------------------
    pcs.profile(True)
    l0 = bg.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier(ws)
        ev0.record(stream)
        for _ in range(args.steps):
            step_device()
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
    launches = bg.kernel_launches() - l0
    prof = pcs.profile_read()
    pcs.profile(False)
    ms = max_over_ranks(ws, ev0.elapsed_time(ev1), device=f"cuda:{local}")
    value = throughput(ws, args.steps, ms)

    # ---- timed region: host buffers through the C ABI ----------------------
    for _ in range(2):
        step_host()
    torch.cuda.synchronize()
    barrier(ws)
    ev0.record(stream)
    for _ in range(args.steps):
        proof = step_host()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    ms_e2e = max_over_ranks(ws, ev0.elapsed_time(ev1), device=f"cuda:{local}")
    e2e = throughput(ws, args.steps, ms_e2e)

    if rank != 0:
        return
    Q = pcs.num_queries()
    d2h = len(proof) + 48 * n + 16
    h2d = 16 * (1 << n) + 16 * n + 8 * Q
    total_ms_classes = sum(v[0] for k, v in prof.items() if k != "encode_last")

    # The trait route: eval of host data with no commitment (bf_eval_data) and
    # the caller-driven open session (one host round trip per round, the
    # caller's challenger), beside the device-transcript open.
    trait = None
    if ws == 1 and not args.no_extras:
        trait = run_trait_route(bg, torch, pcs, dev, evals, point)

    peaks, peak_kind = load_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    num_sms = bg.device_info(local)["num_sms"]
    batched = served = sweep = sumcheck = verify = latency = tuned = prime_res = wide = None
    if ws == 1 and not args.no_extras:
        latency = run_latency(bg, torch, local, log2_c)
        tuned = run_autotune(bg, torch, local, log2_c)
        batched = run_batched(bg, torch, local, log2_c)
        served = run_served(bg, local, log2_c)
        sweep = run_commit_sweep(bg, torch, local)
        sumcheck = run_sumcheck(bg, torch, local)
        verify = run_verify(bg, local, log2_c)
        prime_res = run_prime(bg, torch, local)
        wide = run_binary_wide(bg, torch, local)
    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        t = cpu_step_oracle(n, log2_c)
        cpu = {"value": 1.0 / t, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"one full commit+eval+open at 2^{n} (C++ restatement of the reference CPU path, "
                         "all host threads; the Rust reference cannot be built here)"}
        if served is not None:
            served["cpu_baseline"] = served_cpu_reference(log2_c, served["size_range"])
    clocks = clk.summary()
    sm_mhz = clocks.get("sm_mhz") or 2070.0

    # Roofline of the dominant kernel: the last NTT pass (ntt_reg_kernel<true>),
    # which also hashes the codeword leaves and the first folded-codeword leaves.
    # Algorithmic bytes per codeword pair: 32 read + 32 written (the pair) + three
    # 32-byte digests (two codeword leaves, one folded-codeword leaf) = 160 B.
    c = 1 << log2_c
    pairs = (c << n) // 2
    last_ms, last_launches = prof["encode_last"]
    last_avg_s = last_ms / 1e3 / max(last_launches, 1)
    achieved = 160.0 * pairs / last_avg_s / 1e9 if last_avg_s > 0 else None
    tr = load_traffic("ntt_last_pass_traffic.json")
    traffic = tr["bytes_per_pair"] * pairs if tr and tr.get("bytes_per_pair") else None
    alu_last = None
    if tr and tr.get("alu_thread_inst_per_pair") and last_avg_s > 0:
        alu_last = tr["alu_thread_inst_per_pair"] * pairs / last_avg_s / (64.0 * num_sms * sm_mhz * 1e6)
    # second: the Merkle levels (level_kernel + subtree + top: Keccak of 64-byte nodes)
    tree_ms, tree_scopes = prof["tree"]
    nodes = tree_nodes(n, log2_c) * args.steps
    tr2 = load_traffic()
    perms_per_s = (nodes / (tree_ms / 1e3)) if tree_ms else None
    alu_peak = 64.0 * num_sms * sm_mhz * 1e6 / KECCAK_ALU
    level = {"kernel": "level_kernel+subtree_kernel+tree_top_kernel (Merkle levels)",
             "achieved_gbs": 96.0 * nodes / (tree_ms / 1e3) / 1e9 if tree_ms else None,
             "traffic_bytes_per_node": tr2.get("bytes_per_node") if tr2 else None,
             "keccak_perms_per_s": perms_per_s, "alu_frac": (perms_per_s / alu_peak) if perms_per_s else None}
    step_bytes = algorithmic_bytes(n, log2_c)
    floor_ms = proof_floor_ms(n, log2_c, sm_mhz, num_sms)
    ms_step = ms / args.steps
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "gf2^128+keccak-u64", "data": "synthetic (SplitMix64 seed = rank)",
        "config": workload_config(args),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": {0: "ntt_pass_kernel<true>", 1: "ntt_reg_kernel<true>",
                                2: "ntt_last_ws_kernel"}.get(pcs.tune["ntt_kind"], "?")
                               + ": last NTT pass + codeword and first folded-codeword leaf hashes "
                                 "(160 algorithmic B per codeword pair)",
                     "launch_ms": last_avg_s * 1e3, "share_of_step": last_ms / max(total_ms_classes, 1e-9),
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "alu_frac": alu_last,
                     "note": "integer-ALU bound (Keccak-f), not HBM bound: alu_frac = ALU-pipe instructions "
                             "(ncu count per pair) over 64 per clock per SM at the sampled clock"},
        "roofline_levels": level,
        "step_roofline": {"algorithmic_bytes": step_bytes, "hbm_frac": step_bytes / (ms_step / 1e3) / 1e9 / peak,
                          "instruction_floor_ms": floor_ms, "floor_frac": floor_ms / ms_step},
        "kernel_ms_per_step": {k: round(v[0] / args.steps, 3) for k, v in prof.items()},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": ms_e2e / args.steps},
        "clocks": clocks,
        "gpu_launches": launches,
        "proof_bytes": len(proof),
    }
    # compact extras last: a log that keeps only the end of a long line still holds them
    if trait:
        line["trait_route"] = trait
    if sweep:
        line["commit_sweep"] = {"cols": ["num_vars", "blowup", "ms", "algorithmic_gbs", "keccak_gperm_s"],
                                "rows": [[r["num_vars"], r["blowup"], round(r["ms"], 2), round(r["algorithmic_gbs"], 1),
                                          round(r["keccak_perms_per_s"] / 1e9, 2)] for r in sweep]}
    if latency:
        line["latency_by_size"] = latency
    if tuned:
        line["autotune"] = tuned
    if sumcheck:
        line["sumcheck"] = {"cols": ["k", "num_vars", "ms"],
                            "rows": [[r["k"], r["num_vars"], round(r["ms"], 3)] for r in sumcheck]}
    if verify:
        line["verify"] = {"workload": verify["workload"], "gpu_proofs_per_s": round(verify["gpu_proofs_per_s"]),
                          "cpu_proofs_per_s": round(verify["cpu_baseline"]["proofs_per_s"]),
                          "cpu_cores": verify["cpu_baseline"]["cores"], "speedup": round(verify["speedup"], 1)}
    if wide:
        line["binary_wide"] = wide
    if prime_res:
        line["prime"] = prime_res
    if batched:
        mc = batched["multi_column"]
        line["batched"] = {"workload": batched["workload"],
                           "plain_proofs_per_s": round(batched["plain_proofs_per_s"], 1),
                           "batched_proofs_per_s": round(batched["batched_proofs_per_s"], 1),
                           "speedup": round(batched["speedup"], 3), "identical": batched["proofs_identical"],
                           "floor_s": round(batched["floor_s"], 4), "batched_s": round(batched["batched_s"], 4),
                           "batched_over_floor": round(batched["batched_over_floor"], 3),
                           "small_jobs_le_2^16": {k: (round(v, 4) if isinstance(v, float) else v)
                                                  for k, v in batched["small_jobs"].items()},
                           "multi_column_polys_per_s": round(mc["polys_per_s"], 1)}
    if served:
        sc = served.get("cpu_baseline") or {}
        line["served"] = {"workload": served["workload"],
                          "capacity_proofs_per_s": round(served["capacity_proofs_per_s"], 1),
                          "levels": [[lv["offered_load"], round(lv["achieved_proofs_per_s"], 1), round(lv["p50_ms"], 1),
                                      round(lv["p99_ms"], 1)] for lv in served["levels"]],
                          "levels_cols": ["offered_load", "proofs_per_s", "p50_ms", "p99_ms"],
                          "cpu_service_p50_ms": round(sc["service_p50_ms"], 1) if sc else None,
                          "cpu_service_p99_ms": round(sc["service_p99_ms"], 1) if sc else None,
                          "cpu_cores": sc.get("cores")}
    print(json.dumps(line), flush=True)


def run_trait_route(bg, torch, pcs, dev, evals, point, reps=3):
    """The calls a Rust PolyCommitScheme binding makes (poly-commit/src/lib.rs:
    29-50): eval of host data that has no commitment, and open driven round
    by round by the caller's own challenger (bf_open_start/round/challenge/
    final/finish), beside the device-transcript open on the same commitment."""
    comm = pcs.commit_device(dev.data_ptr(), keep=dev)
    ch = bg.GenericChallenger.keccak256()
    ch.observe(comm.root)
    vals = pcs.eval(evals, point)  # host rows, copied in
    ch.observe_ext_slice(vals)
    pe = [bg.PolyEvals(vals, point)]
    ref = pcs.open(comm, pe, ch.clone())
    assert pcs.open_session(comm, pe[0]).prove(ch.clone()) == ref

    def timed(f):
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            f()
            torch.cuda.synchronize()
            ts.append(1e3 * (time.perf_counter() - t))
        return sorted(ts)[len(ts) // 2]

    out = {"eval_host_data_ms": timed(lambda: pcs.eval(evals, point)),
           "eval_commitment_ms": timed(lambda: pcs.eval(pcs.data(comm), point)),
           "open_device_transcript_ms": timed(lambda: pcs.open(comm, pe, ch.clone())),
           "open_session_ms": timed(lambda: pcs.open_session(comm, pe[0]).prove(ch.clone())),
           "identical": True}
    comm.free()
    return {k: (round(v, 3) if isinstance(v, float) else v) for k, v in out.items()}


if __name__ == "__main__":
    main()
