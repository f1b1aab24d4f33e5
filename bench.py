#!/usr/bin/env python
"""Benchmark of the BYO hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload dynamic|static] [--policy m20|learned|...]

Workloads (synthetic: seeded RMAT a=.57 b=.19 c=.19 d=.05, symmetrised,
deduplicated, no self loops; the reference publishes no dataset for them):
  dynamic  packed-memory-array container on RMAT n=2^22, 2^26 draws.  One step
           = insert one batch of 10^7 uniform (src,dst) pairs, symmetrised
           (2*10^7 directed keys, unsorted), BFS from 10, Connectivity,
           PageRank (eps 1e-6, at most 20 iterations), remove the same batch.
           The batch is the same every step, as in the reference's
           Batch_insert_runner (benchmarks/run_unweighted.h:781-893), so the
           state seen by the traversals repeats exactly.
  static   the same RMAT graph in the CSR container; BFS + CC + PageRank.

The metric is BASELINE's composite; `value` is the step's edge operations per
second in G/s: BFS traversed edges (undirected, Graph500 convention) + CC
edges (undirected) + PageRank directed edges x iterations + inserted and
removed directed keys.  The per-component rates are in `components`.

`value` is measured with the graph and the batch resident in HBM (device
API, CUDA events on the library's stream); `e2e` runs the same step through
the public host API with the batch in pinned host memory and every result
(parents, labels, ranks) copied back to the host inside the timed region.
Under torchrun (N > 1) every rank runs an independent replica (the path does
not shard in this build): weak scaling, value = all ranks' work / max time.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "BFS/PR/CC GTEPS + insert edges/s at 1 GB300, learned vs m/20 policy, bit-exact"
UNIT = "G edge-ops/s (BFS+CC traversed edges, PR edges x iters, inserted+removed keys)"
LG_N, DRAWS, SEED, SRC = 22, 1 << 26, 1, 10
BATCH, BATCH_SEED = 10_000_000, 1001
PR_EPS, PR_ITERS = 1e-6, 20
L2_BYTES = 126 * 1024 * 1024
POLICIES = {"m20": 0, "learned": 1, "push": 2, "pull": 3, "blocked": 4, "m20_blocked": 5}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for name, val in zip(names, f[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ peaks
def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_table():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


# ------------------------------------------------------------------ algorithmic bytes
def pr_iteration_bytes(n, m, nslots):
    # ids 4 B/slot + FP32 p_div gather 4 B/edge + offsets 8(n+1) + deg 4n
    # + p_curr read 4n + p_next write 4n + p_div write 4n
    return 4 * nslots + 4 * m + 8 * (n + 1) + 16 * n


def bfs_bytes(n, reached_deg_sum, reached):
    # neighbour ids of reached vertices once, offsets once, lp write per reached
    # vertex, parent array written once
    return 4 * reached_deg_sum + 8 * (n + 1) + 8 * reached + 4 * n


# ------------------------------------------------------------------ our arm
def run_ours(args, rank, world, local_rank):
    import torch
    import byo_gb300 as byo
    from byo_gb300 import _abi
    L = _abi.lib()
    torch.cuda.set_device(local_rank)
    ctx = byo.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    dynamic = args.workload == "dynamic"
    container = "pma" if dynamic else "csr"
    t0 = time.time()
    G = byo.Graph.generate(ctx, "rmat", seed=SEED, lg_n=LG_N, draws=DRAWS, container=container)
    n, m0 = G.N(), G.M()
    log("graph: n=%d m=%d container=%s built in %.2fs" % (n, m0, container, time.time() - t0))
    from byo_gb300 import policy as learned
    have_net = learned.load_default(ctx)
    if args.policy == "auto":
        args.policy = "learned" if have_net else "m20"
    policy = POLICIES[args.policy]
    if args.policy == "learned":
        _abi.check(L.byo_ctx_set_update_policy(ctx.h, _abi.UPDATE_LEARNED), ctx.h)
    dev = torch.device("cuda", local_rank)
    B = 2 * BATCH
    keys = torch.empty(B, dtype=torch.int64, device=dev)
    if dynamic:
        _abi.check(L.byo_gen_uniform_keys_device(ctx.h, BATCH_SEED, n, BATCH, keys.data_ptr()), ctx.h)
    parent = torch.empty(n, dtype=torch.int32, device=dev)
    label = torch.empty(n, dtype=torch.int32, device=dev)
    pr = torch.empty(n, dtype=torch.float64, device=dev)
    ctx.synchronize()
    ch = ctypes.c_uint64(0)
    rounds = ctypes.c_uint32(0)
    it = ctypes.c_uint32(0)
    l1 = ctypes.c_double(0)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]

    def step(record):
        with torch.cuda.stream(stream):
            if record:
                ev[0].record(stream)
            if dynamic:
                _abi.check(L.byo_graph_insert_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)),
                           ctx.h)
            if record:
                ev[1].record(stream)
            _abi.check(L.byo_bfs_device(G.h, SRC, parent.data_ptr(), None, policy, ctypes.byref(rounds)),
                       ctx.h)
            if record:
                ev[2].record(stream)
            _abi.check(L.byo_cc_device(G.h, label.data_ptr()), ctx.h)
            if record:
                ev[3].record(stream)
            _abi.check(L.byo_pagerank_device(G.h, PR_EPS, PR_ITERS, 0, pr.data_ptr(), ctypes.byref(it),
                                             ctypes.byref(l1)), ctx.h)
            if record:
                ev[4].record(stream)
            if dynamic:
                _abi.check(L.byo_graph_remove_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)),
                           ctx.h)
            if record:
                ev[5].record(stream)

    # warm-up; the last warm-up step's state equals every timed step's
    for _ in range(args.warmup):
        step(False)
    ctx.synchronize()
    deg_t = torch.from_numpy(G.degrees().astype(np.int64))
    # units of one step (state at traversal time: after the insert)
    if dynamic:
        _abi.check(L.byo_graph_insert_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)
        m_trav = G.M()
        deg_t = torch.from_numpy(G.degrees().astype(np.int64))
        nslots = G.nslots()
        _abi.check(L.byo_bfs_device(G.h, SRC, parent.data_ptr(), None, policy, ctypes.byref(rounds)), ctx.h)
        _abi.check(L.byo_graph_remove_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)
    else:
        m_trav, nslots = m0, m0
        _abi.check(L.byo_bfs_device(G.h, SRC, parent.data_ptr(), None, policy, ctypes.byref(rounds)), ctx.h)
    ctx.synchronize()
    reached_mask = (parent.cpu() != -1)
    reached = int(reached_mask.sum())
    bfs_edges = int(deg_t[reached_mask].sum())
    pr_iters = it.value or PR_ITERS
    units = {"bfs": bfs_edges / 2, "cc": m_trav / 2, "pr": m_trav * pr_iters,
             "insert": B if dynamic else 0, "remove": B if dynamic else 0}
    total_units = sum(units.values())

    # timed region
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    ctx.kernel_timing("*")
    launches0 = ctx.launches
    clocks = ClockSampler(local_rank)
    clocks.start()
    comp_ms = np.zeros(5)
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for _ in range(args.steps):
        step(True)
        stream.synchronize()
        for i in range(5):
            comp_ms[i] += ev[i].elapsed_time(ev[i + 1])
    t_end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed_ms = t_start.elapsed_time(t_end)
    launches = ctx.launches - launches0
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([elapsed_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
        dist.barrier()

    # per-kernel shares over the timed region
    tags = ["bfs_push", "bfs_pull", "bfs_blocked", "cc_finish", "pr_pull", "tc_intersect", "sort_scatter",
            "pma_merge", "pma_redistribute"]
    ktimes = {t: ctx.kernel_time(t) for t in tags}
    ctx.kernel_timing(None)
    dom = max(tags, key=lambda t: ktimes[t][1])
    peak, peak_kind = measured_peaks()
    roof = {"bound": "hbm", "peak": peak, "unit": "GB/s", "kernel": dom, "peak_source": peak_kind}
    if dom == "pr_pull":
        # one PageRank iteration = k_pr_units + k_pr_combine (both tagged pr_pull)
        per_iter = pr_iteration_bytes(n, m_trav, nslots)
        launches_dom, ms_dom = ktimes[dom]
        iters_total = pr_iters * args.steps
        achieved = per_iter * iters_total / (ms_dom / 1e3) / 1e9
        roof.update({"kernel": "pr_pull (k_pr_units + k_pr_combine, per iteration)", "achieved": achieved,
                     "frac": achieved / peak, "algorithmic_bytes_per_launch": per_iter,
                     "avg_launch_ms": ms_dom / max(iters_total, 1), "launches": launches_dom,
                     "iterations": iters_total})
    elif dom.startswith("bfs"):
        byts = bfs_bytes(n, bfs_edges, reached) * args.steps
        ms_bfs = sum(ktimes[t][1] for t in tags if t.startswith("bfs"))
        achieved = byts / (ms_bfs / 1e3) / 1e9
        roof.update({"achieved": achieved, "frac": achieved / peak, "kernel": "bfs (push+pull+blocked)"})
    else:
        roof.update({"achieved": None, "frac": None})
    tr = traffic_table().get(dom)
    roof["traffic"] = tr.get("bytes_per_launch") if tr else None
    roof["kernel_ms_share"] = {t: round(ktimes[t][1] / max(elapsed_ms, 1e-9), 4) for t in tags if ktimes[t][0]}

    step_ms = elapsed_ms / args.steps
    value = world * total_units / (step_ms / 1e3) / 1e9
    comp = comp_ms / args.steps
    components = {
        "bfs_gteps": units["bfs"] / (comp[1] / 1e3) / 1e9,
        "cc_gteps": units["cc"] / (comp[2] / 1e3) / 1e9,
        "pr_gteps": units["pr"] / (comp[3] / 1e3) / 1e9,
        "bfs_ms": comp[1], "cc_ms": comp[2], "pr_ms": comp[3], "pr_iters": pr_iters,
        "bfs_rounds": rounds.value,
    }
    if dynamic:
        components.update({"insert_edges_per_s": B / (comp[0] / 1e3), "remove_edges_per_s": B / (comp[4] / 1e3),
                           "insert_ms": comp[0], "remove_ms": comp[4]})

    # the learned policy against the m/20 rule (and in-place merge) on the
    # same state, same GPU: BFS and the update pair, median of 5
    if have_net:
        components["policy_compare"] = compare_policies(L, _abi, ctx, G, keys, B, parent, dynamic, torch, stream)

    # end to end through the public host API
    e2e = run_e2e(args, byo, G, ctx, torch, dynamic, keys, B, n, policy, total_units, world, dev)

    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 ids / fp32-kahan pagerank (fp64 residual)",
        "data": "synthetic (seeded RMAT, no dataset)",
        "config": {"workload": "config[1] dynamic PMA: RMAT 2^22, 2^26 draws, batch 1e7 pairs" if dynamic
                   else "static CSR: RMAT 2^22, 2^26 draws",
                   "n": n, "m": m_trav, "batch_pairs": BATCH if dynamic else 0, "bfs_src": SRC,
                   "pr_eps": PR_EPS, "pr_max_iters": PR_ITERS, "policy": args.policy,
                   "parallelism": "replicas x%d" % world,
                   "l2": "inputs larger than L2 (graph %.0f MB > 126 MB)" % ((8 * n + 4 * nslots) / 1e6)},
        "components": components, "roofline": roof, "e2e": e2e, "gpu_launches": launches,
        "clocks": clk,
    }
    return res, ctx, G


def compare_policies(L, _abi, ctx, G, keys, B, parent, dynamic, torch, stream):
    ch = ctypes.c_uint64(0)
    r = ctypes.c_uint32(0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        ts = []
        for _ in range(5):
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    out = {}
    for name, pol in (("m20", POLICIES["m20"]), ("learned", POLICIES["learned"])):
        out["bfs_ms_" + name] = timed(lambda: _abi.check(L.byo_bfs_device(G.h, SRC, parent.data_ptr(), None, pol,
                                                                          ctypes.byref(r)), ctx.h))
    if dynamic:
        for name, up in (("merge", _abi.UPDATE_MERGE), ("learned", _abi.UPDATE_LEARNED)):
            _abi.check(L.byo_ctx_set_update_policy(ctx.h, up), ctx.h)

            def pair():
                _abi.check(L.byo_graph_insert_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)
                _abi.check(L.byo_graph_remove_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)
            out["update_pair_ms_" + name] = timed(pair)
        _abi.check(L.byo_ctx_set_update_policy(ctx.h, _abi.UPDATE_LEARNED), ctx.h)
    return out


def run_e2e(args, byo, G, ctx, torch, dynamic, keys, B, n, policy, total_units, world, dev):
    host_keys = torch.empty(B, dtype=torch.int64, pin_memory=True)
    host_keys.copy_(keys.cpu()) if dynamic else None
    hk = host_keys.numpy().view(np.uint64)
    par = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    lab = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    prv = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()

    def step():
        if dynamic:
            G.insert_batch(hk)
        byo.BFS(G, SRC, policy=policy, out=par)
        byo.SimpleUnionAsync(G, out=lab)
        byo.PageRank(G, PR_EPS, PR_ITERS, out=prv)
        if dynamic:
            G.remove_batch(hk)

    step()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / args.steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([dt], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt = float(t.item())
    return {"value": world * total_units / dt / 1e9, "unit": UNIT,
            "h2d_bytes_per_step": (2 * 8 * B) if dynamic else 0,
            "d2h_bytes_per_step": 4 * n + 4 * n + 8 * n, "ms_per_step": dt * 1e3}


# ------------------------------------------------------------------ CPU (oracle) legs
def cpu_setup(dynamic):
    from oracle import oracle as O
    O.build()
    s, d = O.rmat_edges(SEED, LG_N, DRAWS)
    off, nb = O.build_csr(1 << LG_N, s, d)
    del s, d
    keys = None
    if dynamic:
        us, ud = O.uniform_pairs(BATCH_SEED, 1 << LG_N, BATCH)
        keys = O.keys_from_pairs(us, ud)
    return O, off, nb, keys


def cpu_step(O, off, nb, keys, store):
    """One step of the workload on the CPU restatement; returns (units, ms per phase)."""
    t = [time.perf_counter()]
    if keys is not None:
        store.insert_batch(keys)
        off, nb = store.export_csr()
    t.append(time.perf_counter())
    par, _ = O.bfs(off, nb, SRC)
    t.append(time.perf_counter())
    O.cc(off, nb)
    t.append(time.perf_counter())
    _, iters, _ = O.pagerank(off, nb, PR_EPS, PR_ITERS)
    t.append(time.perf_counter())
    if keys is not None:
        store.remove_batch(keys)
    t.append(time.perf_counter())
    m = len(nb)
    deg = np.diff(off.astype(np.int64))
    reached = par != O.NONE
    units = deg[reached].sum() / 2 + m / 2 + m * iters + (2 * len(keys) if keys is not None else 0)
    return float(units), np.diff(t) * 1e3


def run_reference(args, dynamic):
    O, off, nb, keys = cpu_setup(dynamic)
    store = O.Store(off, nb) if dynamic else None
    threads = O.num_threads()
    for _ in range(args.warmup):
        cpu_step(O, off, nb, keys, store)
    tot_units, tot_s = 0.0, 0.0
    for _ in range(args.steps):
        u, ph = cpu_step(O, off, nb, keys, store)
        tot_units += u
        tot_s += ph.sum() / 1e3
    value = tot_units / tot_s / 1e9
    sample = "full steps of the workload on the oracle port (OpenMP), %d threads" % threads
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_s * 1e3 / args.steps, "higher_is_better": True,
            "impl": "reference",
            "config": {"workload": "config[1] dynamic PMA: RMAT 2^22, 2^26 draws, batch 1e7 pairs" if dynamic
                       else "static CSR: RMAT 2^22, 2^26 draws"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "data": "synthetic (seeded RMAT, no dataset)"}


def cpu_baseline_sample(dynamic):
    O, off, nb, keys = cpu_setup(dynamic)
    store = O.Store(off, nb) if dynamic else None
    u, ph = cpu_step(O, off, nb, keys, store)
    secs = ph.sum() / 1e3
    return {"value": u / secs / 1e9, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": "one full step of the same workload on the oracle port (OpenMP, %d threads), %.1f s"
                      % (O.num_threads(), secs),
            "phase_ms": {k: float(v) for k, v in zip(["insert", "bfs", "cc", "pr", "remove"], ph)}}


# ------------------------------------------------------------------ main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dynamic", choices=["dynamic", "static"])
    ap.add_argument("--policy", default="auto", choices=sorted(POLICIES) + ["auto"],
                    help="auto: the committed learned network if present, else m20")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warm-up raised to 3 steps")
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dynamic = args.workload == "dynamic"

    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, dynamic)), flush=True)
        return 0

    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    res, ctx, G = run_ours(args, rank, world, local_rank)
    G.close()
    ctx.close()
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            res["cpu_baseline"] = cpu_baseline_sample(dynamic)
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
