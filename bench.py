#!/usr/bin/env python
"""Benchmark of the BYO hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload dynamic|static|mixed|multi|scale|families|map|bytepd|stream|tc]
                    [--container pma|vos|pcsr] [--policy m20|learned|...]

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
  mixed    64-source BFS groups interleaved with update batches (RMAT 2^24).
  multi    64-source BFS groups only.
  scale    RMAT 2^26 / 2^30 draws and ER 2^26: BFS, CC, PageRank precisions, TC.
  families learned policy vs m/20 on RMAT, ER, a grid and Chung-Lu.
  map      Test_Map and Test_Map_Remote (every remote width) on the dynamic
           workload's graph, CSR and PMA.
  bytepd   the dynamic workload's graph in the byte-PD compressed format,
           decoded into a CSR on the GPU.
  stream   200 small update batches inserted then removed on the mixed
           workload's PMA through byo_graph_update_stream, against one call
           per batch.
  tc       triangle counting (degree ordered) on RMAT n=2^22, average degree
           32, CSR: one count per step.
--container vos runs the dynamic step on the vector of per-vertex runs,
--container pcsr on the packed CSR (sentinels and neighbour ids in one array).

The metric is the composite of BFS, CC, PageRank and update rates; `value` is the step's edge operations per
second in G/s: BFS traversed edges (undirected, Graph500 convention) + CC
edges (undirected) + PageRank directed edges x iterations + inserted and
removed directed keys.  The per-component rates are in `components`.

`value` is measured with the graph and the batch resident in HBM (device
API, CUDA events on the library's stream); `e2e` runs the same step through
the public host API with the batch in pinned host memory and every result
(parents, labels, ranks) copied back to the host inside the timed region.
Under torchrun (N > 1) every rank runs an independent replica (the path does
not shard): weak scaling, value = all ranks' work / max time.
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


# ------------------------------------------------------------------ replicas
def max_over_ranks(x, world):
    """The largest of every rank's x (each rank is an independent replica;
    the job's time is its slowest rank's).  nccl reduces on the device,
    gloo on the host."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, world, ms_max):
    """Whole-job rate: every rank's units over the slowest rank's time (G/s)."""
    return world * units_per_rank / (ms_max / 1e3) / 1e9


# ------------------------------------------------------------------ NVTX
def nvtx_push(torch, name):
    """Marks the timed region (ncu --nvtx --nvtx-include "timed/" captures it alone)."""
    try:
        torch.cuda.nvtx.range_push(name)
        return True
    except Exception:
        return False


def nvtx_pop(torch, pushed):
    if pushed:
        torch.cuda.nvtx.range_pop()


class nvtx_range:
    """A named range inside the timed region, one per component of a step
    (ncu --nvtx --nvtx-include "timed/pagerank/" captures PageRank's launches)."""

    def __init__(self, torch, name, on=True):
        self.torch, self.name, self.on, self.pushed = torch, name, on, False

    def __enter__(self):
        if self.on:
            self.pushed = nvtx_push(self.torch, self.name)

    def __exit__(self, *exc):
        nvtx_pop(self.torch, self.pushed)


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


def cc_bytes(n, m):
    # one pass over the edges (ids), offsets once, labels read + written once
    return 4 * m + 8 * (n + 1) + 8 * n


# bytes a merge reads and writes per element of a touched leaf: the PMA's
# 4-byte src and dst read and written; the PCSR's 4-byte slot read and written
# (its sentinel bits add 1/4 B); the vector of runs reports no touched leaves
ENTRY_BYTES = {"pma": 16, "pcsr": 8.25, "vos": 8}


def update_bytes(B, touched_entries, container="pma"):
    # 8-byte keys read + written once for the sort, and every element of
    # every leaf the merge touches read + written once
    return 16 * B + ENTRY_BYTES[container] * touched_entries


def dynamic_config(dynamic, container, n, m):
    """The workload description both arms print (same keys and values)."""
    return {"workload": ("dynamic %s: RMAT 2^22, 2^26 draws, batch 1e7 pairs" % container.upper()) if dynamic
            else "static CSR: RMAT 2^22, 2^26 draws",
            "n": int(n), "m": int(m), "batch_pairs": BATCH if dynamic else 0, "bfs_src": SRC,
            "pr_eps": PR_EPS, "pr_max_iters": PR_ITERS, "rmat": [0.57, 0.19, 0.19], "seed": SEED,
            "batch_seed": BATCH_SEED if dynamic else None,
            "l2": "inputs larger than L2 (RMAT 2^22 graph > 126 MB)"}


# ------------------------------------------------------------------ parity against the oracle
def parity_selfcheck(byo, L, _abi, ctx, G, keys, B, policy, dynamic, O, off0, nb0, okeys):
    """The headline workload's outputs against the oracle, on the state the
    timed steps see (before the timed region): container contents before the
    batch, after the insert and after the remove; BFS parents and levels and
    CC labels bit for bit; PageRank (FP32-Kahan) L1 against the FP64 oracle.
    Returns the parity block and the oracle's sorted-set store holding the
    contents after the remove (the batch's pairs that were already edges are
    gone then, in both), for the batch sweep."""
    ch = ctypes.c_uint64(0)
    go, gn = G.export_csr()
    contents = bool(np.array_equal(go, off0) and np.array_equal(gn, nb0))
    so, sn = off0, nb0
    st = None
    if dynamic:
        st = O.Store(off0, nb0)
        _abi.check(L.byo_graph_insert_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)
        contents &= int(ch.value) == st.insert_batch(okeys)
        so, sn = st.export_csr()
        go, gn = G.export_csr()
        contents &= bool(np.array_equal(go, so) and np.array_equal(gn, sn))
    par, lev = byo.BFS(G, SRC, policy=policy, levels=True)
    opar, olev = O.bfs(so, sn, SRC)
    bfs_ok = bool(np.array_equal(par, opar) and np.array_equal(lev, olev))
    lab = byo.SimpleUnionAsync(G)
    cc_ok = bool(np.array_equal(lab, O.cc(so, sn)))
    p, it, _ = byo.PageRank(G, PR_EPS, PR_ITERS, info=True)
    op, oit, _ = O.pagerank(so, sn, PR_EPS, PR_ITERS)
    l1 = float(np.abs(p - op).sum())
    del so, sn
    if dynamic:
        _abi.check(L.byo_graph_remove_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)
        contents &= int(ch.value) == st.remove_batch(okeys)
        so, sn = st.export_csr()
        go, gn = G.export_csr()
        contents &= bool(np.array_equal(go, so) and np.array_equal(gn, sn))
    block = {"contents": contents, "bfs": bfs_ok, "cc": cc_ok, "pr_l1": l1, "pr_l1_bound": 1e-6,
             "pr_iters": [int(it), int(oit)],
             "checked": "before the timed region, on the state the timed steps see: contents (sorted adjacency) "
                        "before the batch, after the insert and after the remove, and the changed-key counts; "
                        "BFS(%d) parents + levels and CC labels after the insert, bit-exact; PageRank "
                        "FP32-Kahan vs the FP64 oracle, L1 over all vertices" % SRC}
    block["ok"] = bool(contents and bfs_ok and cc_ok and l1 <= 1e-6)
    return block, st


SWEEP_SIZES = (1_000, 100_000, 10_000_000)
SWEEP_ROUNDS = 10


def batch_sweep(byo, L, _abi, ctx, G, torch, stream, dev, n, policy, O, st):
    """BASELINE's dynamic-container schedule (Batch_insert_runner,
    benchmarks/run_unweighted.h:781-893): for each batch size b in 1e3, 1e5,
    1e7 pairs, rounds 0..10 (round 0 untimed), each inserting a fresh batch
    of b uniform pairs, symmetrised (2b directed keys, unsorted), then
    removing it.  Insert and remove are timed on the device (CUDA events on
    the library's stream around the device-API call); after every batch,
    outside the timing, the contents and changed-key count are compared with
    the oracle's sorted-set store `st` (which holds the container's contents
    on entry) and BFS(10) parents and CC labels with the oracle's answers on
    those contents."""
    ch = ctypes.c_uint64(0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out, checks, failures = {}, 0, []
    kbuf = torch.empty(2 * max(SWEEP_SIZES), dtype=torch.int64, device=dev)
    t_verify = 0.0
    for b in SWEEP_SIZES:
        tag = "1e%d" % (len(str(b)) - 1)
        ins_ms, rem_ms, upd_bytes = [], [], [0.0, 0.0]
        for r in range(SWEEP_ROUNDS + 1):
            seed = 50_000 + 1000 * len(str(b)) + r
            _abi.check(L.byo_gen_uniform_keys_device(ctx.h, seed, n, b, kbuf.data_ptr()), ctx.h)
            us, ud = O.uniform_pairs(seed, n, b)
            okeys = O.keys_from_pairs(us, ud)
            for phase in (1, 0):
                ctx.synchronize()
                with torch.cuda.stream(stream):
                    e0.record(stream)
                    fn = L.byo_graph_insert_batch_device if phase else L.byo_graph_remove_batch_device
                    _abi.check(fn(G.h, kbuf.data_ptr(), 2 * b, 0, ctypes.byref(ch)), ctx.h)
                    e1.record(stream)
                e1.synchronize()
                ms = e0.elapsed_time(e1)
                if r > 0:
                    (ins_ms if phase else rem_ms).append(ms)
                    upd_bytes[1 - phase] += update_bytes(2 * b, G.last_update_stats()["touched_entries"], G.container)
                # verification, outside the timing
                tv = time.perf_counter()
                ok = int(ch.value) == (st.insert_batch(okeys) if phase else st.remove_batch(okeys))
                so, sn = st.export_csr()
                go, gn = G.export_csr()
                ok &= bool(np.array_equal(go, so) and np.array_equal(gn, sn))
                del go, gn
                opar, _ = O.bfs(so, sn, SRC)
                ok &= bool(np.array_equal(byo.BFS(G, SRC, policy=policy), opar))
                ok &= bool(np.array_equal(byo.SimpleUnionAsync(G), O.cc(so, sn)))
                del so, sn
                checks += 1
                if not ok:
                    failures.append("%s %s round %d" % ("insert" if phase else "remove", tag, r))
                t_verify += time.perf_counter() - tv
        ti, tr = float(np.mean(ins_ms)), float(np.mean(rem_ms))
        out["insert_edges_per_s_" + tag] = 2 * b / (ti / 1e3)
        out["remove_edges_per_s_" + tag] = 2 * b / (tr / 1e3)
        out["insert_ms_" + tag] = ti
        out["remove_ms_" + tag] = tr
        out["insert_hbm_gbs_" + tag] = upd_bytes[0] / (sum(ins_ms) / 1e3) / 1e9
        out["remove_hbm_gbs_" + tag] = upd_bytes[1] / (sum(rem_ms) / 1e3) / 1e9
    out["verified_batches"] = checks
    out["verify_failures"] = failures
    out["verified"] = not failures
    out["how"] = ("%d rounds (+1 untimed) per size, a fresh seeded batch of uniform pairs each round, symmetrised, "
                  "insert then remove; edges/s = directed keys (2 x pairs) / device time of the call (sort + merge + "
                  "view upkeep, as the reference times insert_batch, run_unweighted.h:832-835); every batch, timed "
                  "and untimed, verified against the oracle outside the timing: contents, changed count, BFS(%d) "
                  "parents, CC labels (%.1f s of checking); hbm_gbs = (16 B per key + 16 B (PMA) or 8.25 B "
                  "(PCSR) per element of every touched leaf) / time" % (SWEEP_ROUNDS, SRC, t_verify))
    return out


# ------------------------------------------------------------------ our arm
def run_ours(args, rank, world, local_rank):
    import torch
    import byo_gb300 as byo
    from byo_gb300 import _abi
    L = _abi.lib()
    torch.cuda.set_device(local_rank)
    ctx = byo.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    if args.pr_launches == "stream":
        _abi.check(L.byo_ctx_set_pagerank_graphs(ctx.h, 0), ctx.h)
    dynamic = args.workload == "dynamic"
    container = args.container if dynamic else "csr"
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
    # parity of this exact workload against the oracle, before any timing
    parity, ostore, O = None, None, None
    if rank == 0 and not args.no_parity:
        t0 = time.time()
        O, off0, nb0, okeys = cpu_setup(dynamic)
        parity, ostore = parity_selfcheck(byo, L, _abi, ctx, G, keys, B, policy, dynamic, O, off0, nb0, okeys)
        del off0, nb0, okeys
        parity["seconds"] = round(time.time() - t0, 1)
        log("parity vs oracle: %s" % json.dumps(parity))
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
                with nvtx_range(torch, "insert", record):
                    _abi.check(L.byo_graph_insert_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)),
                               ctx.h)
            if record:
                ev[1].record(stream)
            with nvtx_range(torch, "bfs", record):
                _abi.check(L.byo_bfs_device(G.h, SRC, parent.data_ptr(), None, policy, ctypes.byref(rounds)),
                           ctx.h)
            if record:
                ev[2].record(stream)
            with nvtx_range(torch, "cc", record):
                _abi.check(L.byo_cc_device(G.h, label.data_ptr()), ctx.h)
            if record:
                ev[3].record(stream)
            with nvtx_range(torch, "pagerank", record):
                _abi.check(L.byo_pagerank_device(G.h, PR_EPS, PR_ITERS, 0, pr.data_ptr(), ctypes.byref(it),
                                                 ctypes.byref(l1)), ctx.h)
            if record:
                ev[4].record(stream)
            if dynamic:
                with nvtx_range(torch, "remove", record):
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
        nslots = m_trav  # the read-only algorithms traverse the PMA's compact snapshot
        _abi.check(L.byo_bfs_device(G.h, SRC, parent.data_ptr(), None, policy, ctypes.byref(rounds)), ctx.h)
        _abi.check(L.byo_graph_remove_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)
    else:
        m_trav, nslots = m0, m0
        _abi.check(L.byo_bfs_device(G.h, SRC, parent.data_ptr(), None, policy, ctypes.byref(rounds)), ctx.h)
    ctx.synchronize()
    reached_mask = (parent.cpu() != -1)
    reached = int(reached_mask.sum())
    bfs_edges = int(deg_t[reached_mask].sum())
    upd_stats = {}
    if dynamic:  # leaves the merge touches (the state repeats every step)
        _abi.check(L.byo_graph_insert_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)
        upd_stats["insert"] = G.last_update_stats()
        _abi.check(L.byo_graph_remove_batch_device(G.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)
        upd_stats["remove"] = G.last_update_stats()
        ctx.synchronize()
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
    pushed = nvtx_push(torch, "timed")
    t_start.record(stream)
    for _ in range(args.steps):
        step(True)
        stream.synchronize()
        for i in range(5):
            comp_ms[i] += ev[i].elapsed_time(ev[i + 1])
    t_end.record(stream)
    torch.cuda.synchronize()
    nvtx_pop(torch, pushed)
    clk = clocks.stop()
    elapsed_ms = t_start.elapsed_time(t_end)
    launches = ctx.launches - launches0
    elapsed_ms = max_over_ranks(elapsed_ms, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()

    # per-kernel shares over the timed region
    tags = ["bfs_push", "bfs_pull", "bfs_blocked", "cc_finish", "pr_pull", "tc_intersect", "sort_scatter",
            "pma_merge", "pma_redistribute", "pcsr_merge", "pcsr_redistribute", "pcsr_compact"]
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
    if dom == "pr_pull":
        # second roof: the device's random one-word gather rate from a table
        # the size of PageRank's FP32 p/deg array (L2-resident)
        gr = ctypes.c_double(0)
        _abi.check(L.byo_gather_roof(ctx.h, 4 * n, ctypes.byref(gr)), ctx.h)
        got = m_trav * pr_iters * args.steps / (ktimes[dom][1] / 1e3)
        roof["gather_roof"] = {"unit": "G gathers/s", "peak": gr.value / 1e9, "achieved": got / 1e9,
                               "frac": got / gr.value if gr.value else None, "table_bytes": 4 * n,
                               "how": "byo_gather_roof: uniform random 4-byte loads from a table of 4n bytes, "
                                      "16 in flight per thread, best of 5 launches (CUDA events); achieved = "
                                      "directed edges x iterations / PageRank kernel time"}
    tr = traffic_table().get(dom)
    roof["traffic"] = tr.get("bytes_per_launch") if tr else None
    roof["kernel_ms_share"] = {t: round(ktimes[t][1] / max(elapsed_ms, 1e-9), 4) for t in tags if ktimes[t][0]}

    step_ms = elapsed_ms / args.steps
    value = replica_value(total_units, world, step_ms)
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

    # a roofline fraction per component, from each phase's device time
    # (CUDA events around the call) and its algorithmic bytes
    def frac(byts, ms):
        gbs = byts / (ms / 1e3) / 1e9
        return {"achieved_gbs": gbs, "frac": gbs / peak, "algorithmic_bytes": byts, "ms": ms}
    per = {"bfs": frac(bfs_bytes(n, bfs_edges, reached), comp[1]),
           "cc": frac(cc_bytes(n, m_trav), comp[2]),
           "pr": frac(pr_iteration_bytes(n, m_trav, nslots) * pr_iters, comp[3])}
    if dynamic:
        per["insert"] = frac(update_bytes(B, upd_stats["insert"]["touched_entries"], container), comp[0])
        per["remove"] = frac(update_bytes(B, upd_stats["remove"]["touched_entries"], container), comp[4])
        per["insert"]["touched_leaves"] = upd_stats["insert"]["touched_leaves"]
        per["insert"]["touched_entries"] = upd_stats["insert"]["touched_entries"]
        per["remove"]["touched_leaves"] = upd_stats["remove"]["touched_leaves"]
        per["remove"]["touched_entries"] = upd_stats["remove"]["touched_entries"]
    roof["per_component"] = per
    roof["per_component_bytes"] = ("bfs 4*sum(deg of reached) + 8(n+1) + 8*reached + 4n (includes the PMA snapshot "
                                   "rebuild in its time); cc one pass 4m + 8(n+1) + 8n; pr per iteration 4m + 4m + "
                                   "8(n+1) + 16n; insert/remove 16 B per key + per element of every touched leaf "
                                   "16 B (PMA) or 8.25 B (PCSR)")

    # the learned policy against the m/20 rule (and in-place merge) on the
    # same state, same GPU: BFS and the update pair, median of 5
    if have_net:
        components["policy_compare"] = compare_policies(L, _abi, ctx, G, keys, B, parent, dynamic, torch, stream)

    # end to end through the public host API
    e2e = run_e2e(args, byo, G, ctx, torch, dynamic, keys, B, n, policy, total_units, world, dev)

    # the same step on the packed CSR container
    if dynamic and container == "pma" and rank == 0 and not args.no_pcsr:
        t0 = time.time()
        components["pcsr"] = pcsr_compare(args, byo, L, _abi, ctx, torch, stream, keys, B, policy, G, parent, label,
                                          pr, total_units, peak)
        log("pcsr arm: %.1f s" % (time.time() - t0))

    # BASELINE's batch-size sweep with verification after every batch
    if dynamic and ostore is not None and not args.no_sweep:
        t0 = time.time()
        components["batch_sweep"] = batch_sweep(byo, L, _abi, ctx, G, torch, stream, dev, n, policy, O, ostore)
        log("batch sweep: %.1f s" % (time.time() - t0))

    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 ids / fp32-kahan pagerank (fp64 residual)",
        "data": "synthetic (seeded RMAT, no dataset)",
        "config": dynamic_config(dynamic, container, n, m_trav),
        "policy": args.policy, "parallelism": "replicas x%d" % world,
        "parity": parity,
        "components": components, "roofline": roof, "e2e": e2e, "gpu_launches": launches,
        "clocks": clk,
    }
    return res, ctx, G


def pcsr_compare(args, byo, L, _abi, ctx, torch, stream, keys, B, policy, G, parent, label, pr, total_units,
                 peak):
    """The dynamic step on the packed CSR container (run_pcsr.cc's layout:
    per-vertex sentinels and neighbour ids in one packed array) built from the
    same RMAT draws: its contents after the insert must equal the headline
    container's (whose contents the oracle checked), then W warm-up and K timed
    steps of the same insert, BFS, CC, PageRank, remove with CUDA events per
    phase on the library's stream."""
    P = byo.Graph.generate(ctx, "rmat", seed=SEED, lg_n=LG_N, draws=DRAWS, container="pcsr")
    ch = ctypes.c_uint64(0)
    rounds, it, l1 = ctypes.c_uint32(0), ctypes.c_uint32(0), ctypes.c_double(0)

    def ins(g):
        _abi.check(L.byo_graph_insert_batch_device(g.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)

    def rem(g):
        _abi.check(L.byo_graph_remove_batch_device(g.h, keys.data_ptr(), B, 0, ctypes.byref(ch)), ctx.h)

    ins(P)
    ins(G)
    po, pn = P.export_csr()
    go, gn = G.export_csr()
    same = bool(np.array_equal(po, go) and np.array_equal(pn, gn))
    del po, pn, go, gn
    nslots_after_insert = P.nslots()
    rem(P)
    rem(G)
    ins(P)
    st_ins = P.last_update_stats()
    rem(P)
    st_rem = P.last_update_stats()
    ctx.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]

    def step(record):
        with torch.cuda.stream(stream):
            if record:
                ev[0].record(stream)
            ins(P)
            if record:
                ev[1].record(stream)
            _abi.check(L.byo_bfs_device(P.h, SRC, parent.data_ptr(), None, policy, ctypes.byref(rounds)), ctx.h)
            if record:
                ev[2].record(stream)
            _abi.check(L.byo_cc_device(P.h, label.data_ptr()), ctx.h)
            if record:
                ev[3].record(stream)
            _abi.check(L.byo_pagerank_device(P.h, PR_EPS, PR_ITERS, 0, pr.data_ptr(), ctypes.byref(it),
                                             ctypes.byref(l1)), ctx.h)
            if record:
                ev[4].record(stream)
            rem(P)
            if record:
                ev[5].record(stream)

    for _ in range(args.warmup):
        step(False)
    ctx.synchronize()
    comp = np.zeros(5)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        step(True)
        stream.synchronize()
        for i in range(5):
            comp[i] += ev[i].elapsed_time(ev[i + 1])
    t1.record(stream)
    torch.cuda.synchronize()
    step_ms = t0.elapsed_time(t1) / args.steps
    comp /= args.steps

    def frac(byts, ms):
        gbs = byts / (ms / 1e3) / 1e9
        return {"achieved_gbs": gbs, "frac": gbs / peak, "algorithmic_bytes": byts, "ms": ms}

    out = {"same_contents_as_pma": same, "value": total_units / (step_ms / 1e3) / 1e9, "ms_per_step": step_ms,
           "insert_ms": comp[0], "bfs_ms": comp[1], "cc_ms": comp[2], "pr_ms": comp[3], "remove_ms": comp[4],
           "insert_edges_per_s": B / (comp[0] / 1e3), "remove_edges_per_s": B / (comp[4] / 1e3),
           "insert_roofline": frac(update_bytes(B, st_ins["touched_entries"], "pcsr"), comp[0]),
           "remove_roofline": frac(update_bytes(B, st_rem["touched_entries"], "pcsr"), comp[4]),
           "slots": nslots_after_insert, "container_bytes": int(nslots_after_insert * 4.125),
           "pma_container_bytes": int(G.nslots() * 8),
           "how": "same step and units as the headline; value = the headline's edge operations per step / this "
                  "step's device time; BFS includes the snapshot rebuild (k_pcsr_compact)"}
    P.close()
    return out


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
    dt = max_over_ranks(dt, world)
    return {"value": world * total_units / dt / 1e9, "unit": UNIT,
            "h2d_bytes_per_step": (2 * 8 * B) if dynamic else 0,
            "d2h_bytes_per_step": 4 * n + 4 * n + 8 * n, "ms_per_step": dt * 1e3}


# ------------------------------------------------------------------ mixed queries + updates
MIXED_LG, MIXED_DRAWS, MIXED_SEED = 24, 8 << 24, 5
MIXED_QUERIES, MIXED_BATCHES = 16, 8
MIXED_METRIC = "mixed stream: 64-source BFS queries + insert/delete batches (log-uniform 1e2-1e6 pairs)"
MIXED_UNIT = "G edge-ops/s (BFS traversed edges over all sources + inserted and removed keys)"


def mixed_ops(seed):
    """One step's op list: MIXED_QUERIES query groups and MIXED_BATCHES insert
    batches, each deleted later in the same step, in a seeded random order;
    batch sizes (pairs, symmetrised on insert) log-uniform in [1e2, 1e6]."""
    rng = np.random.default_rng(seed)
    sizes = np.round(10.0 ** rng.uniform(2, 6, MIXED_BATCHES)).astype(np.int64)
    ops = ([("Q", i) for i in range(MIXED_QUERIES)] + [("I", j) for j in range(MIXED_BATCHES)]
           + [("D", j) for j in range(MIXED_BATCHES)])
    order = [ops[i] for i in rng.permutation(len(ops))]
    pos = {op: i for i, op in enumerate(order)}
    for j in range(MIXED_BATCHES):
        a, b = pos[("I", j)], pos[("D", j)]
        if b < a:
            order[a], order[b] = order[b], order[a]
    return order, sizes


def mixed_sources(deg, seed):
    rng = np.random.default_rng(seed + 17)
    nz = np.nonzero(deg)[0]
    return [np.ascontiguousarray(rng.choice(nz, 64), np.uint32) for _ in range(MIXED_QUERIES)]


def size_bin(b):
    return "1e%d-1e%d" % (int(np.log10(max(b, 1))), int(np.log10(max(b, 1))) + 1)


def run_mixed(args, rank, world, local_rank):
    import torch
    import byo_gb300 as byo
    from byo_gb300 import _abi
    from byo_gb300 import policy as learned
    L = _abi.lib()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = byo.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    t0 = time.time()
    G = byo.Graph.generate(ctx, "rmat", seed=MIXED_SEED, lg_n=MIXED_LG, draws=MIXED_DRAWS, container="pma")
    n, m0 = G.N(), G.M()
    log("mixed: n=%d m=%d built in %.2fs" % (n, m0, time.time() - t0))
    if learned.load_default(ctx):
        _abi.check(L.byo_ctx_set_update_policy(ctx.h, _abi.UPDATE_LEARNED), ctx.h)
    t0 = time.time()
    tuning = G.autotune(bfs=False, multi=True, trials=3)
    tune_s = time.time() - t0
    order, sizes = mixed_ops(MIXED_SEED)
    deg = G.degrees()
    qsrc = mixed_sources(deg, MIXED_SEED)
    bkeys = []
    for j, b in enumerate(sizes):
        k = torch.empty(2 * int(b), dtype=torch.int64, device=dev)
        _abi.check(L.byo_gen_uniform_keys_device(ctx.h, MIXED_SEED * 1000 + j, n, int(b), k.data_ptr()), ctx.h)
        bkeys.append(k)
    levels = torch.empty(64 * n, dtype=torch.int32, device=dev)
    ch = ctypes.c_uint64(0)
    rounds = ctypes.c_uint32(0)

    def run_op(op):
        kind, i = op
        if kind == "Q":
            _abi.check(L.byo_bfs_multi_device(G.h, qsrc[i].ctypes.data, 64, levels.data_ptr(),
                                              ctypes.byref(rounds)), ctx.h)
        elif kind == "I":
            k = bkeys[i]
            _abi.check(L.byo_graph_insert_batch_device(G.h, k.data_ptr(), k.numel(), 0, ctypes.byref(ch)), ctx.h)
        else:
            k = bkeys[i]
            _abi.check(L.byo_graph_remove_batch_device(G.h, k.data_ptr(), k.numel(), 0, ctypes.byref(ch)), ctx.h)

    def step(lat):
        for op in order:
            a = time.perf_counter()
            run_op(op)
            lat.append((op, time.perf_counter() - a))

    for _ in range(args.warmup):
        step([])
    ctx.synchronize()
    # traversed edges of every query group on the step's start state
    deg_t = torch.from_numpy(deg.astype(np.int64)).to(dev)
    q_edges = []
    for i in range(MIXED_QUERIES):
        run_op(("Q", i))
        ctx.synchronize()
        reached = (levels.view(64, n) != -1)
        q_edges.append(float((reached.to(torch.int64) * deg_t).sum().item()) / 2)
    upd_keys = float(sum(2 * 2 * int(b) for b in sizes))
    units = sum(q_edges) + upd_keys
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    ctx.kernel_timing("*")
    launches0 = ctx.launches
    clocks = ClockSampler(local_rank)
    clocks.start()
    lat = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pushed = nvtx_push(torch, "timed")
    e0.record(stream)
    t_host = time.perf_counter()
    for _ in range(args.steps):
        step(lat)
    e1.record(stream)
    torch.cuda.synchronize()
    nvtx_pop(torch, pushed)
    t_host = time.perf_counter() - t_host
    clk = clocks.stop()
    launches = ctx.launches - launches0
    elapsed_ms = e0.elapsed_time(e1)
    ms_launches, ms_kernel = ctx.kernel_time("bfs_multi")
    ctx.kernel_timing(None)
    elapsed_ms = max_over_ranks(elapsed_ms, world)
    step_ms = elapsed_ms / args.steps
    qlat = np.array([x for (op, x) in lat if op[0] == "Q"]) * 1e3
    ulat = {}
    for (op, x) in lat:
        if op[0] != "Q":
            ulat.setdefault(size_bin(int(sizes[op[1]])), []).append(x * 1e3)
    allu = np.array([x for v in ulat.values() for x in v])
    peak, peak_kind = measured_peaks()
    nslots = m0  # the compact snapshot
    # lower bound of one 64-source launch: levels written once, the adjacency
    # read once, the three mask arrays (seen, F, N) read and written once
    ms_bytes = 4 * 64 * n + 4 * nslots + 8 * (n + 1) + 6 * 8 * n
    per_launch_ms = ms_kernel / max(ms_launches, 1)
    achieved = ms_bytes / (per_launch_ms / 1e3) / 1e9
    res = {
        "metric": MIXED_METRIC, "value": world * units / (step_ms / 1e3) / 1e9, "unit": MIXED_UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32 ids, u64 source masks", "data": "synthetic (seeded RMAT, uniform update pairs)",
        "config": {"workload": "mixed: RMAT 2^24 avg deg 16 (2^27 draws) PMA; per step %d query groups of 64 "
                               "seeded sources + %d insert batches deleted later in the step" %
                               (MIXED_QUERIES, MIXED_BATCHES),
                   "n": n, "m": m0, "batch_pairs": [int(b) for b in sizes], "tuning": tuning,
                   "autotune_s": tune_s, "parallelism": "replicas x%d" % world,
                   "l2": "inputs larger than L2 (graph %.0f MB)" % ((8 * n + 4 * nslots) / 1e6)},
        "components": {
            "queries_per_s": 64 * MIXED_QUERIES / (step_ms / 1e3),
            "update_keys_per_s": upd_keys / (step_ms / 1e3),
            "query_latency_ms": {"p50": float(np.percentile(qlat, 50)), "p99": float(np.percentile(qlat, 99)),
                                 "mean": float(qlat.mean())},
            "update_latency_ms": {"p50": float(np.percentile(allu, 50)), "p99": float(np.percentile(allu, 99))},
            "update_latency_ms_by_pairs": {k: {"p50": float(np.percentile(v, 50)), "p99": float(np.percentile(v, 99)),
                                               "count": len(v)} for k, v in sorted(ulat.items())},
            "query_traversed_edges_per_group": float(np.mean(q_edges)),
            "host_ms_per_step": t_host * 1e3 / args.steps,
            "bfs_multi_kernel_ms": per_launch_ms,
        },
        "roofline": {"bound": "hbm", "kernel": "k_ms_bfs (one 64-source traversal)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": ms_bytes, "avg_launch_ms": per_launch_ms,
                     "traffic": (traffic_table().get("bfs_multi") or {}).get("bytes_per_launch"),
                     "kernel_ms_share": round(ms_kernel / max(elapsed_ms, 1e-9), 4)},
        "gpu_launches": launches, "clocks": clk,
    }
    # the same step as one mixed stream (byo_graph_mixed_stream_device): runs
    # of queries and batches of up to 4096 keys drained by one persistent
    # kernel; larger batches finished on the host between launches
    res["components"]["one_launch"] = mixed_one_launch(args, L, _abi, ctx, G, torch, stream, dev, n, order,
                                                       sizes, bkeys, qsrc, units)
    # end to end: batches from pinned host memory, every query's levels back to the host
    hk = []
    for k in bkeys:
        h = torch.empty(k.numel(), dtype=torch.int64, pin_memory=True)
        h.copy_(k.cpu())
        hk.append(h.numpy().view(np.uint64))
    hlev = torch.empty(64 * n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)

    def e2e_op(op):
        kind, i = op
        if kind == "Q":
            _abi.check(L.byo_bfs_multi(G.h, qsrc[i].ctypes.data, 64, hlev.ctypes.data, None), ctx.h)
        elif kind == "I":
            G.insert_batch(hk[i])
        else:
            G.remove_batch(hk[i])

    for op in order:
        e2e_op(op)
    torch.cuda.synchronize()
    a = time.perf_counter()
    for _ in range(args.steps):
        for op in order:
            e2e_op(op)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - a) / args.steps
    res["e2e"] = {"value": world * units / dt / 1e9, "unit": MIXED_UNIT,
                  "h2d_bytes_per_step": int(upd_keys * 8),
                  "d2h_bytes_per_step": 4 * 64 * n * MIXED_QUERIES, "ms_per_step": dt * 1e3}
    return res, ctx, G


def mixed_one_launch(args, L, _abi, ctx, G, torch, stream, dev, n, order, sizes, bkeys, qsrc, units):
    ops, offs, srcs, kparts = [], [0], [], []
    for kind, i in order:
        if kind == "Q":
            ops.append(_abi.OP_QUERY)
            srcs.append(qsrc[i])
        else:
            ops.append(_abi.OP_INSERT if kind == "I" else _abi.OP_REMOVE)
            kparts.append(bkeys[i])
        offs.append(offs[-1] + (0 if kind == "Q" else bkeys[i].numel()))
    keys = torch.cat(kparts)
    offs = np.ascontiguousarray(offs, np.uint64)
    opc = np.ascontiguousarray(ops, np.uint8)
    srcv = np.ascontiguousarray(np.concatenate(srcs), np.uint32)
    nq = len(srcs)
    levels = torch.empty(nq * 64 * n, dtype=torch.int32, device=dev)
    ch = np.zeros(len(ops), np.uint64)
    t = np.zeros(2 * len(ops), np.uint64)
    torch.cuda.synchronize()

    def step():
        _abi.check(L.byo_graph_mixed_stream_device(G.h, keys.data_ptr(), offs.ctypes.data, opc.ctypes.data, len(ops),
                                                   srcv.ctypes.data, 64, levels.data_ptr(), ch.ctypes.data,
                                                   t.ctypes.data), ctx.h)

    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launches
    qlat = []
    e0.record(stream)
    for _ in range(args.steps):
        step()
        tt = t.reshape(-1, 2)
        qlat += [(tt[i, 1] - tt[i, 0]) / 1e6 for i in range(len(ops)) if ops[i] == _abi.OP_QUERY]
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    tt = t.reshape(-1, 2)
    in_kernel = [i for i in range(len(ops)) if tt[i, 1] > 0]
    qlat = np.array(qlat)
    del levels
    return {"value": units / (ms / 1e3) / 1e9, "unit": MIXED_UNIT, "ms_per_step": ms,
            "query_latency_ms": {"p50": float(np.percentile(qlat, 50)), "p99": float(np.percentile(qlat, 99)),
                                 "mean": float(qlat.mean())},
            "ops_in_kernel": len(in_kernel), "ops": len(ops),
            "launches_per_step": (ctx.launches - launches0) / args.steps,
            "how": "the step's %d ops through byo_graph_mixed_stream_device: queries and batches of <= 4096 keys "
                   "run inside one persistent kernel (query latency = its device start/end times); larger "
                   "batches on the host path between launches" % len(ops)}


def run_multi(args, rank, world, local_rank):
    """64-source BFS only: one step = one query group of 64 seeded sources
    (the groups of the mixed workload, in turn) on the PMA graph."""
    import torch
    import byo_gb300 as byo
    from byo_gb300 import _abi
    L = _abi.lib()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = byo.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    lg = args.lg or MIXED_LG
    G = byo.Graph.generate(ctx, "rmat", seed=MIXED_SEED, lg_n=lg, draws=8 << lg, container="pma")
    n, m0 = G.N(), G.M()
    tuning = G.autotune(bfs=False, multi=True, trials=3) if not args.no_autotune else G.tuning()
    deg = G.degrees()
    qsrc = mixed_sources(deg, MIXED_SEED)
    levels = torch.empty(64 * n, dtype=torch.int32, device=dev)
    deg_t = torch.from_numpy(deg.astype(np.int64)).to(dev)
    r = ctypes.c_uint32(0)

    def q(i):
        _abi.check(L.byo_bfs_multi_device(G.h, qsrc[i % MIXED_QUERIES].ctypes.data, 64, levels.data_ptr(),
                                          ctypes.byref(r)), ctx.h)

    for i in range(args.warmup):
        q(i)
    edges = []
    for i in range(args.steps):
        q(i)
        ctx.synchronize()
        edges.append(float(((levels.view(64, n) != -1).to(torch.int64) * deg_t).sum().item()) / 2)
    torch.cuda.synchronize()
    ctx.kernel_timing("*")
    launches0 = ctx.launches
    clocks = ClockSampler(local_rank)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pushed = nvtx_push(torch, "timed")
    e0.record(stream)
    for i in range(args.steps):
        q(i)
    e1.record(stream)
    torch.cuda.synchronize()
    nvtx_pop(torch, pushed)
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    kl, kms = ctx.kernel_time("bfs_multi")
    ctx.kernel_timing(None)
    rounds_log = [(x["round"], x["mode"], x["frontier"], round(x["ms"], 3)) for x in ctx.last_rounds()]
    peak, peak_kind = measured_peaks()
    nslots = m0  # the compact snapshot
    ms_bytes = 4 * 64 * n + 4 * nslots + 8 * (n + 1) + 6 * 8 * n
    per = kms / max(kl, 1)
    units = sum(edges)
    res = {"metric": "64-source bit-lane BFS, traversed edges over all sources", "value": units / (ms / 1e3) / 1e9,
           "unit": "G traversed edges/s (sum over the 64 sources, Graph500 count)", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u64 source masks", "data": "synthetic (seeded RMAT)",
           "config": {"workload": "64-source BFS on RMAT 2^%d, %d draws (PMA)" % (lg, 8 << lg), "n": n, "m": m0,
                      "tuning": tuning, "rounds": rounds_log},
           "roofline": {"bound": "hbm", "kernel": "k_ms_bfs", "achieved": ms_bytes / (per / 1e3) / 1e9, "peak": peak,
                        "unit": "GB/s", "frac": ms_bytes / (per / 1e3) / 1e9 / peak, "peak_source": peak_kind,
                        "algorithmic_bytes_per_launch": ms_bytes, "avg_launch_ms": per,
                        "traffic": (traffic_table().get("bfs_multi") or {}).get("bytes_per_launch")},
           "gpu_launches": ctx.launches - launches0, "clocks": clk}
    return res, ctx, G


# ------------------------------------------------------------------ neighbour maps
MAP_WIDTHS = (0, 1, 2, 4, 8, 16, 32)


def map_remote_array(n, width, seed):
    """Map_Remote_runner's array (run_unweighted.h:50-126): n zeros of `width`
    bytes with one seeded random entry set to 1 (width 0: a bitmap)."""
    one = int(np.random.default_rng(seed).integers(0, n))
    if width == 0:
        a = np.zeros((n + 63) // 64, np.uint64)
        a[one >> 6] = np.uint64(1) << np.uint64(one & 63)
    elif width <= 8:
        a = np.zeros(n, {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[width])
        a[one] = 1
    else:
        a = np.zeros((n, width // 8), np.uint64)
        a[one, 0] = 1
    return a


def run_map(args, rank, world, local_rank):
    """Map and Map_Remote (run_all's first applications, run_unweighted.h:
    27-126, 943-957) on the dynamic workload's graph in both containers: one
    step = Test_Map and Test_Map_Remote for every width, on the CSR and on the
    PMA (its leaves scanned as they lie)."""
    import torch
    import byo_gb300 as byo
    from byo_gb300 import _abi
    L = _abi.lib()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = byo.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    graphs = [byo.Graph.generate(ctx, "rmat", seed=SEED, lg_n=LG_N, draws=DRAWS, container=c) for c in ("csr", "pma")]
    n, m0 = graphs[0].N(), graphs[0].M()
    remotes = {w: torch.from_numpy(map_remote_array(n, w, 100 + w).view(np.uint8).copy()).to(dev) for w in MAP_WIDTHS}
    out = ctypes.c_uint64(0)
    sums = {}

    def step(record=False):
        for G, name in zip(graphs, ("csr", "pma")):
            _abi.check(L.byo_map_sum(G.h, ctypes.byref(out)), ctx.h)
            if record:
                sums[name + "/map"] = out.value
            for w in MAP_WIDTHS:
                _abi.check(L.byo_map_remote_device(G.h, remotes[w].data_ptr(), w, ctypes.byref(out)), ctx.h)
                if record:
                    sums["%s/remote%d" % (name, w)] = out.value

    for i in range(args.warmup):
        step(record=i == 0)
    torch.cuda.synchronize()
    ctx.kernel_timing("map")
    launches0 = ctx.launches
    clocks = ClockSampler(local_rank)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pushed = nvtx_push(torch, "timed")
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    nvtx_pop(torch, pushed)
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    kl, kms = ctx.kernel_time("map")
    ctx.kernel_timing(None)
    # per kind: time of one launch (device) and its rate
    per_kind = {}
    for G, name in zip(graphs, ("csr", "pma")):
        for w in (None,) + MAP_WIDTHS:
            ctx.kernel_timing("map")
            for _ in range(3):
                if w is None:
                    _abi.check(L.byo_map_sum(G.h, ctypes.byref(out)), ctx.h)
                else:
                    _abi.check(L.byo_map_remote_device(G.h, remotes[w].data_ptr(), w, ctypes.byref(out)), ctx.h)
            cl, cms = ctx.kernel_time("map")
            ctx.kernel_timing(None)
            t = cms / max(cl, 1)
            per_kind["%s/%s" % (name, "map" if w is None else "remote%d" % w)] = {
                "ms": round(t, 4), "G_edges_s": round(G.M() / (t / 1e3) / 1e9, 1),
                "slot_GBs": round(4 * G.nslots() / (t / 1e3) / 1e9, 1)}
    peak, peak_kind = measured_peaks()
    edges_per_step = sum(G.M() for G in graphs) * (1 + len(MAP_WIDTHS))
    slot_bytes = sum(4 * G.nslots() for G in graphs) * (1 + len(MAP_WIDTHS))
    per = kms / max(kl, 1)
    avg_bytes = slot_bytes / max(kl / args.steps, 1)
    res = {"metric": "Test_Map + Test_Map_Remote edges/s (run_all's Map applications)",
           "value": edges_per_step * args.steps / (ms / 1e3) / 1e9, "unit": "G edges/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u32 ids, u64 sums", "data": "synthetic (seeded RMAT)",
           "config": {"workload": "map: RMAT 2^%d, %d draws, CSR and PMA, widths %s" % (LG_N, DRAWS, list(MAP_WIDTHS)),
                      "n": n, "m": m0, "per_kind": per_kind, "sums": sums},
           "roofline": {"bound": "hbm", "kernel": "k_map_sum", "achieved": avg_bytes / (per / 1e3) / 1e9,
                        "peak": peak, "unit": "GB/s", "frac": avg_bytes / (per / 1e3) / 1e9 / peak,
                        "peak_source": peak_kind, "algorithmic_bytes_per_launch": avg_bytes, "avg_launch_ms": per,
                        "traffic": None},
           "gpu_launches": ctx.launches - launches0, "clocks": clk}
    for G in graphs[1:]:
        G.close()
    return res, ctx, graphs[0]


def map_cpu_sample():
    """The oracle's Test_Map / Test_Map_Remote on the CSR of the same graph
    (OpenMP, all host threads): one pass of each kind."""
    O, off, nb, _ = cpu_setup(False)
    n = len(off) - 1
    remotes = {w: map_remote_array(n, w, 100 + w) for w in MAP_WIDTHS}
    passes, secs = 0, 0.0
    while secs < 3.0:  # whole passes, at least 3 s of CPU work
        t0 = time.time()
        for w in (None,) + MAP_WIDTHS:
            if w is None:
                O.map_sum(off, nb)
            else:
                O.map_remote(off, nb, remotes[w], w)
        secs += time.time() - t0
        passes += 1
    m = len(nb)
    return {"value": m * (1 + len(MAP_WIDTHS)) * passes / secs / 1e9, "unit": "G edges/s",
            "cores": O.num_threads(), "kind": "port",
            "sample": "%d passes of Test_Map and Test_Map_Remote per width on the CSR (oracle port, OpenMP, "
                      "%d threads), %.1f s" % (passes, O.num_threads(), secs)}


# ------------------------------------------------------------------ triangle counting
def tc_dag_bytes(off, nb):
    """Algorithmic bytes of one degree-ordered TC (4 per id of both out-lists
    per DAG edge, Triangle.h:167-204 with intersect.h:72-151), from the CSR on
    the host: rank by (degree, id), DAG edges point to the higher rank."""
    n = len(off) - 1
    deg = np.diff(off.astype(np.int64))
    order = np.lexsort((np.arange(n), deg))
    rank = np.empty(n, np.int64)
    rank[order] = np.arange(n)
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    up = rank[nb.astype(np.int64)] > rank[src]
    s, d = src[up], nb.astype(np.int64)[up]
    dplus = np.bincount(s, minlength=n)
    return int(4 * (dplus[s].sum() + dplus[d].sum())), int(len(s))


def run_tc(args, rank, world, local_rank):
    """TriangleCounting (Triangle_degree_ordering) on RMAT 2^22 with average
    degree 32 (the scale workload's TC graph), CSR: one step = one count."""
    import torch
    import byo_gb300 as byo
    from byo_gb300 import _abi
    L = _abi.lib()
    torch.cuda.set_device(local_rank)
    ctx = byo.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    name, desc, spec = TC_GRAPH
    spec = dict(spec)
    kind = spec.pop("kind")
    G = byo.Graph.generate(ctx, kind, container="csr", **spec)
    n, m = G.N(), G.M()
    off, nb = G.export_csr()
    alg_bytes, dag_edges = tc_dag_bytes(off, nb)
    del off, nb
    cnt = ctypes.c_uint64(0)
    for _ in range(args.warmup):
        _abi.check(L.byo_triangle_count(G.h, ctypes.byref(cnt)), ctx.h)
    torch.cuda.synchronize()
    launches0 = ctx.launches
    clocks = ClockSampler(local_rank)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pushed = nvtx_push(torch, "timed")
    e0.record(stream)
    for _ in range(args.steps):
        _abi.check(L.byo_triangle_count(G.h, ctypes.byref(cnt)), ctx.h)
    e1.record(stream)
    torch.cuda.synchronize()
    nvtx_pop(torch, pushed)
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    launches = ctx.launches - launches0
    # end to end: the host API from a host CSR (graph upload included)
    offh, nbh = G.export_csr()
    t0 = time.perf_counter()
    H = byo.Graph.from_csr(ctx, offh, nbh)
    c2 = byo.Triangle_degree_ordering(H)
    e2e_s = time.perf_counter() - t0
    H.close()
    assert c2 == cnt.value
    peak, peak_kind = measured_peaks()
    res = {"metric": "TriangleCounting (degree-ordered) edges/s on RMAT 2^22, average degree 32",
           "value": m / (ms / 1e3) / 1e9, "unit": "G edges/s (directed edges of the graph per count)",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 ids, u64 count",
           "data": "synthetic (seeded RMAT)",
           "config": {"workload": "tc: %s, CSR" % desc, "n": n, "m": m, "dag_edges": dag_edges,
                      "triangles": int(cnt.value), "l2": "graph 513 MB > L2"},
           "roofline": {"bound": "hbm", "kernel": "k_tc_warp + k_tc_block (one count)",
                        "achieved": alg_bytes / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": alg_bytes / (ms / 1e3) / 1e9 / peak, "peak_source": peak_kind,
                        "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": ms, "traffic": None},
           "e2e": {"value": m / e2e_s / 1e9, "unit": "G edges/s (directed edges of the graph per count)",
                   "h2d_bytes_per_step": int(offh.nbytes + nbh.nbytes), "d2h_bytes_per_step": 8},
           "gpu_launches": launches, "clocks": clk}
    return res, ctx, G


def tc_cpu_sample():
    """The oracle's degree-ordered TC (OpenMP, all host threads) on RMAT 2^18
    with average degree 32 (2^22 draws): a bounded sample of the workload."""
    from oracle import oracle as O
    O.build()
    s, d = O.rmat_edges(1, 18, 1 << 22)
    off, nb = O.build_csr(1 << 18, s, d)
    runs, secs = 0, 0.0
    while secs < 3.0:
        t0 = time.time()
        O.triangle_count(off, nb)
        secs += time.time() - t0
        runs += 1
    return {"value": len(nb) * runs / secs / 1e9, "unit": "G edges/s (directed edges of the graph per count)",
            "cores": O.num_threads(), "kind": "port",
            "sample": "%d counts on RMAT 2^18, 2^22 draws (oracle port, OpenMP, %d threads), %.1f s"
                      % (runs, O.num_threads(), secs)}


# ------------------------------------------------------------------ update stream
STREAM_BATCHES, STREAM_SEED = 200, 4242


def stream_batches(n, seed):
    """STREAM_BATCHES symmetrised uniform batches of 10-2000 pairs
    (log-uniform), as Batch_insert_runner's small sizes produce them."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(10), np.log(2000), STREAM_BATCHES)).astype(np.int64)
    out = []
    for k in sizes:
        pairs = rng.integers(0, n, size=(int(k), 2), dtype=np.uint64)
        keys = np.concatenate([(pairs[:, 0] << np.uint64(32)) | pairs[:, 1],
                               (pairs[:, 1] << np.uint64(32)) | pairs[:, 0]])
        out.append(keys[(keys >> np.uint64(32)) != (keys & np.uint64(0xFFFFFFFF))])
    return out


def run_stream(args, rank, world, local_rank):
    """Small update batches, one step = the 200 batches inserted and then
    removed on the mixed workload's PMA (RMAT 2^24): through
    byo_graph_update_stream (one persistent kernel per run of small batches)
    and, for comparison, one byo_graph_insert/remove_batch_device call per
    batch."""
    import torch
    import byo_gb300 as byo
    from byo_gb300 import _abi
    L = _abi.lib()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = byo.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    lg = args.lg or MIXED_LG
    G = byo.Graph.generate(ctx, "rmat", seed=MIXED_SEED, lg_n=lg, draws=8 << lg, container="pma")
    n, m0 = G.N(), G.M()
    bs = stream_batches(n, STREAM_SEED)
    nb = len(bs)
    keys = np.concatenate(bs + bs)
    offs = np.zeros(2 * nb + 1, np.uint64)
    offs[1:] = np.cumsum([len(b) for b in bs + bs])
    ops = np.array([1] * nb + [0] * nb, np.uint8)
    d_keys = torch.from_numpy(keys.view(np.int64)).to(dev)
    changed = np.zeros(2 * nb, np.uint64)
    total_keys = int(offs[-1])

    def stream_step():
        _abi.check(L.byo_graph_update_stream_device(G.h, d_keys.data_ptr(), offs.ctypes.data, ops.ctypes.data,
                                                    2 * nb, changed.ctypes.data), ctx.h)

    ch = ctypes.c_uint64(0)

    def batch_step():
        for i in range(2 * nb):
            f = L.byo_graph_insert_batch_device if ops[i] else L.byo_graph_remove_batch_device
            _abi.check(f(G.h, d_keys.data_ptr() + 8 * int(offs[i]), int(offs[i + 1] - offs[i]), 0, ctypes.byref(ch)),
                       ctx.h)

    for _ in range(args.warmup):
        stream_step()
        batch_step()
    assert G.M() == m0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    launches0 = ctx.launches
    clocks = ClockSampler(local_rank)
    clocks.start()
    pushed = nvtx_push(torch, "timed")
    ms_stream = timed(stream_step)
    nvtx_pop(torch, pushed)
    clk = clocks.stop()
    launches = ctx.launches - launches0
    ms_batch = timed(batch_step)
    assert G.M() == m0
    res = {"metric": "small update batches, keys applied per second (insert then remove, 10-2000 pairs each)",
           "value": total_keys / (ms_stream / 1e3) / 1e9, "unit": "G keys/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_stream, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "u64 keys", "data": "synthetic (seeded RMAT, uniform update pairs)",
           "config": {"workload": "stream: RMAT 2^%d PMA, %d batches of 10-2000 pairs, inserted then removed"
                                  % (lg, nb), "n": n, "m": m0, "keys_per_step": total_keys,
                      "us_per_batch_stream": ms_stream * 1e3 / (2 * nb),
                      "us_per_batch_calls": ms_batch * 1e3 / (2 * nb),
                      "speedup_vs_calls": ms_batch / ms_stream},
           "gpu_launches": launches // max(args.steps, 1), "clocks": clk}
    return res, ctx, G


# ------------------------------------------------------------------ byte-PD graphs
def run_bytepd(args, rank, world, local_rank):
    """Compressed graphs (gbbs/encodings/byte_pd_amortized.h): the dynamic
    workload's graph encoded on the GPU, then one step = decoding the byte-PD
    arrays (host memory, as read from a file) into a CSR on the GPU."""
    import torch
    import byo_gb300 as byo
    torch.cuda.set_device(local_rank)
    ctx = byo.Context(local_rank)
    G = byo.Graph.generate(ctx, "rmat", seed=SEED, lg_n=LG_N, draws=DRAWS)
    n, m = G.N(), G.M()
    ctx.kernel_timing("bytepd_encode")
    bo, dg, data = G.to_bytepd(1000)
    _, enc_ms = ctx.kernel_time("bytepd_encode")
    ctx.kernel_timing(None)
    enc_ms /= 2  # to_bytepd encodes twice (size query, then the bytes)
    for _ in range(args.warmup):
        byo.Graph.from_bytepd(ctx, bo, dg, data).close()
    ctx.kernel_timing("bytepd_decode")
    launches0 = ctx.launches
    clocks = ClockSampler(local_rank)
    clocks.start()
    pushed = nvtx_push(torch, "timed")
    t0 = time.time()
    for _ in range(args.steps):
        H = byo.Graph.from_bytepd(ctx, bo, dg, data)
        H.close()
    wall = (time.time() - t0) / args.steps
    nvtx_pop(torch, pushed)
    clk = clocks.stop()
    kl, kms = ctx.kernel_time("bytepd_decode")
    ctx.kernel_timing(None)
    per = kms / args.steps  # the decode kernels of one step
    peak, peak_kind = measured_peaks()
    nbytes = len(data)
    alg = nbytes + 4 * m + 8 * (n + 1) * 2 + 4 * n  # bytes read, ids written, offsets and degrees
    res = {"metric": "byte-PD decode edges/s (compressed neighbour lists to CSR on the GPU)",
           "value": m / (per / 1e3) / 1e9, "unit": "G edges/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": per, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "u8 varints -> u32 ids", "data": "synthetic (seeded RMAT)",
           "config": {"workload": "byte-PD: RMAT 2^%d, %d draws, block 1000" % (LG_N, DRAWS), "n": n, "m": m,
                      "compressed_bytes": nbytes, "bytes_per_edge": nbytes / max(m, 1),
                      "encode_ms": enc_ms, "decode_ms": per,
                      "note": "value: decode kernel time; e2e: host arrays to a finished CSR graph"},
           "roofline": {"bound": "hbm", "kernel": "k_bpd_decode", "achieved": alg / (per / 1e3) / 1e9, "peak": peak,
                        "unit": "GB/s", "frac": alg / (per / 1e3) / 1e9 / peak, "peak_source": peak_kind,
                        "algorithmic_bytes_per_launch": alg, "avg_launch_ms": per, "traffic": None},
           "e2e": {"value": m / wall / 1e9, "unit": "G edges/s", "h2d_bytes_per_step": int(nbytes + bo.nbytes + dg.nbytes),
                   "d2h_bytes_per_step": 0, "ms_per_step": wall * 1e3},
           "gpu_launches": ctx.launches - launches0, "clocks": clk}
    return res, ctx, G


def bytepd_cpu_sample():
    """The oracle's decode of the same arrays (OpenMP, all host threads)."""
    O, off, nb, _ = cpu_setup(False)
    bo, dg, data = O.bytepd_encode(off, nb, 1000)
    passes, secs = 0, 0.0
    while secs < 3.0:
        t0 = time.time()
        O.bytepd_decode(bo, dg, data, 1000)
        secs += time.time() - t0
        passes += 1
    return {"value": len(nb) * passes / secs / 1e9, "unit": "G edges/s", "cores": O.num_threads(), "kind": "port",
            "sample": "%d decodes of the same byte-PD arrays (oracle port, OpenMP, %d threads), %.1f s"
                      % (passes, O.num_threads(), secs)}


# ------------------------------------------------------------------ scale and graph families
SCALE_GRAPHS = [
    ("rmat26", "RMAT 2^26, 2^30 draws (~2^31 directed)", dict(kind="rmat", seed=1, lg_n=26, draws=1 << 30)),
    ("er26", "ER 2^26, avg degree 32", dict(kind="er", seed=2, n=1 << 26, draws=16 << 26)),
]
FAMILY_GRAPHS = SCALE_GRAPHS + [
    ("grid4096", "grid 4096 x 4096, 4-neighbour", dict(kind="grid", n=4096, draws=4096)),
    ("chung_lu24", "Chung-Lu 2^24, exponent 2.1, avg degree 16", dict(kind="chung_lu", seed=4, n=1 << 24,
                                                                     draws=8 << 24, exponent=2.1)),
]
TC_GRAPH = ("rmat22_deg32", "RMAT 2^22, avg degree 32 (2^26 draws)", dict(kind="rmat", seed=1, lg_n=22,
                                                                         draws=1 << 26))


def _sources(deg, count, seed):
    rng = np.random.default_rng(seed)
    nz = np.nonzero(deg)[0]
    out = [10] if deg[10] else []
    while len(out) < count:
        out.append(int(rng.choice(nz)))
    return out


class _Timer:
    def __init__(self, torch, stream):
        self.torch, self.stream = torch, stream
        self.a = torch.cuda.Event(enable_timing=True)
        self.b = torch.cuda.Event(enable_timing=True)

    def __call__(self, fn, reps=1):
        ts = []
        for _ in range(reps):
            self.a.record(self.stream)
            fn()
            self.b.record(self.stream)
            self.b.synchronize()
            ts.append(self.a.elapsed_time(self.b))
        return float(np.median(ts))


def run_scale(args, rank, world, local_rank):
    """Config C3: BFS, CC and PageRank (FP32 compensated against FP64) on the
    2^26-vertex RMAT and ER graphs in the CSR container; triangle counting on
    RMAT 2^22 with average degree 32."""
    import torch
    import byo_gb300 as byo
    from byo_gb300 import _abi
    from byo_gb300 import policy as learned
    L = _abi.lib()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = byo.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    timer = _Timer(torch, stream)
    learned.load_default(ctx)
    peak, peak_kind = measured_peaks()
    comps, launches, pr_roof = {}, 0, None
    clocks = ClockSampler(local_rank)
    clocks.start()
    for name, desc, spec in SCALE_GRAPHS:
        spec = dict(spec)
        kind = spec.pop("kind")
        t0 = time.time()
        G = byo.Graph.generate(ctx, kind, container="csr", **spec)
        n, m = G.N(), G.M()
        ctx.synchronize()
        gen_s = time.time() - t0
        deg = G.degrees()
        deg_t = torch.from_numpy(deg.astype(np.int64)).to(dev)
        par = torch.empty(n, dtype=torch.int32, device=dev)
        par2 = torch.empty(n, dtype=torch.int32, device=dev)
        lab = torch.empty(n, dtype=torch.int32, device=dev)
        p32 = torch.empty(n, dtype=torch.float64, device=dev)
        p64 = torch.empty(n, dtype=torch.float64, device=dev)
        pf = torch.empty(n, dtype=torch.float64, device=dev)
        it, l1, r = ctypes.c_uint32(0), ctypes.c_double(0), ctypes.c_uint32(0)
        launches0 = ctx.launches
        g = {"graph": desc, "n": n, "m": m, "generate_s": gen_s}
        bfs = []
        for src in _sources(deg, 4, 7):
            row = {"src": src}
            for pname, pol in (("m20", _abi.POLICY_M20), ("learned", _abi.POLICY_LEARNED)):
                out = par if pname == "m20" else par2
                _abi.check(L.byo_bfs_device(G.h, src, out.data_ptr(), None, pol, None), ctx.h)  # warm
                row["ms_" + pname] = timer(lambda: _abi.check(L.byo_bfs_device(G.h, src, out.data_ptr(), None, pol,
                                                                                ctypes.byref(r)), ctx.h), 3)
            row["bit_exact"] = bool(torch.equal(par, par2))
            row["edges"] = float((deg_t * (par != -1)).sum().item()) / 2
            row["gteps_m20"] = row["edges"] / row["ms_m20"] / 1e6
            row["gteps_learned"] = row["edges"] / row["ms_learned"] / 1e6
            bfs.append(row)
        g["bfs"] = bfs
        _abi.check(L.byo_cc_device(G.h, lab.data_ptr()), ctx.h)
        g["cc_ms"] = timer(lambda: _abi.check(L.byo_cc_device(G.h, lab.data_ptr()), ctx.h), 3)
        g["cc_gteps"] = m / 2 / g["cc_ms"] / 1e6
        lb = lab.to(torch.int64)
        g["cc_components"] = int((lb == torch.arange(n, device=dev)).sum().item())
        for key, prec, buf in (("fp32_kahan", _abi.PR_FP32_KAHAN, p32), ("fp64", _abi.PR_FP64, p64),
                               ("fp32", _abi.PR_FP32, pf)):
            _abi.check(L.byo_pagerank_device(G.h, 0.0, PR_ITERS, prec, buf.data_ptr(), ctypes.byref(it),
                                             ctypes.byref(l1)), ctx.h)
            ctx.kernel_timing("pr_pull")
            ms = timer(lambda: _abi.check(L.byo_pagerank_device(G.h, 0.0, PR_ITERS, prec, buf.data_ptr(),
                                                                ctypes.byref(it), ctypes.byref(l1)), ctx.h), 3)
            kl, kms = ctx.kernel_time("pr_pull")
            ctx.kernel_timing(None)
            g["pr_" + key] = {"ms": ms, "iters": it.value, "gteps": m * it.value / ms / 1e6,
                              "kernel_ms_per_iter": kms / max(3 * it.value, 1)}
        g["pr_l1_fp32_kahan_vs_fp64"] = float((p32 - p64).abs().sum().item())
        g["pr_l1_fp32_vs_fp64"] = float((pf - p64).abs().sum().item())
        g["pr_sum_fp64"] = float(p64.sum().item())
        per_iter = g["pr_fp32_kahan"]["kernel_ms_per_iter"]
        achieved = pr_iteration_bytes(n, m, G.nslots()) / (per_iter / 1e3) / 1e9
        if pr_roof is None:
            pr_roof = {"bound": "hbm", "kernel": "pr_pull (k_pr_units + k_pr_combine) on " + name,
                       "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "peak_source": peak_kind, "algorithmic_bytes_per_launch": pr_iteration_bytes(n, m, G.nslots()),
                       "avg_launch_ms": per_iter, "traffic": None}
        ms_lev = torch.empty(64 * n, dtype=torch.int32, device=dev)
        srcs64 = np.ascontiguousarray(_sources(deg, 64, 11), np.uint32)
        _abi.check(L.byo_bfs_multi_device(G.h, srcs64.ctypes.data, 64, ms_lev.data_ptr(), None), ctx.h)
        g["bfs64_ms"] = timer(lambda: _abi.check(L.byo_bfs_multi_device(G.h, srcs64.ctypes.data, 64,
                                                                         ms_lev.data_ptr(), None), ctx.h), 2)
        del ms_lev
        launches += ctx.launches - launches0
        comps[name] = g
        G.close()
        del par, par2, lab, p32, p64, pf
        torch.cuda.empty_cache()
    # triangle counting
    name, desc, spec = TC_GRAPH
    spec = dict(spec)
    kind = spec.pop("kind")
    G = byo.Graph.generate(ctx, kind, container="csr", **spec)
    cnt = byo.Triangle_degree_ordering(G)
    tms = timer(lambda: byo.Triangle_degree_ordering(G), 3)
    comps[name] = {"graph": desc, "n": G.N(), "m": G.M(), "triangles": int(cnt), "tc_ms": tms,
                   "tc_edges_per_s": G.M() / tms * 1e3}
    G.close()
    clk = clocks.stop()
    rm = comps["rmat26"]
    bfs_ms = float(np.mean([b["ms_learned"] for b in rm["bfs"]]))
    bfs_edges = float(np.mean([b["edges"] for b in rm["bfs"]]))
    step_ms = bfs_ms + rm["cc_ms"] + rm["pr_fp32_kahan"]["ms"]
    units = bfs_edges + rm["m"] / 2 + rm["m"] * rm["pr_fp32_kahan"]["iters"]
    res = {"metric": "scale: BFS + CC + PageRank (FP32 compensated) edge-ops/s on RMAT 2^26 (2^31 directed)",
           "value": units / step_ms / 1e6, "unit": "G edge-ops/s (BFS traversed + CC + PR edges x iters)",
           "n_gpus": world, "steps": 3, "warmup": 1, "ms_per_step": step_ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u32 ids / fp32-kahan pagerank (fp64 residual)",
           "data": "synthetic (seeded RMAT / ER)", "config": {"workload": "C3 scale (CSR container)",
                                                               "pr_iters": PR_ITERS, "policy": "learned vs m20"},
           "components": comps, "roofline": pr_roof, "gpu_launches": launches, "clocks": clk}
    return res, ctx, None


def run_families(args, rank, world, local_rank):
    """Config C4: the learned policy against the m/20 rule on RMAT, ER, grid
    and Chung-Lu graphs (PMA container): BFS time from four sources each, the
    update pair (insert + remove of 10^6 pairs) with the learned update
    strategy against the in-place merge, outputs compared bit for bit."""
    import torch
    import byo_gb300 as byo
    from byo_gb300 import _abi
    from byo_gb300 import policy as learned
    L = _abi.lib()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = byo.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    timer = _Timer(torch, stream)
    if not learned.load_default(ctx):
        raise SystemExit("no trained policy to compare")
    comps, launches = {}, 0
    ch, r = ctypes.c_uint64(0), ctypes.c_uint32(0)
    clocks = ClockSampler(local_rank)
    clocks.start()
    tot = {"m20": 0.0, "learned": 0.0, "merge": 0.0, "learned_update": 0.0}
    for name, desc, spec in FAMILY_GRAPHS:
        spec = dict(spec)
        kind = spec.pop("kind")
        G = byo.Graph.generate(ctx, kind, container="pma", **spec)
        n, m = G.N(), G.M()
        deg = G.degrees()
        par = torch.empty(n, dtype=torch.int32, device=dev)
        par2 = torch.empty(n, dtype=torch.int32, device=dev)
        launches0 = ctx.launches
        g = {"graph": desc, "n": n, "m": m, "bfs": []}
        for src in _sources(deg, 4, 9):
            row = {"src": src}
            for pname, pol, out in (("m20", _abi.POLICY_M20, par), ("learned", _abi.POLICY_LEARNED, par2)):
                _abi.check(L.byo_bfs_device(G.h, src, out.data_ptr(), None, pol, None), ctx.h)
                row["ms_" + pname] = timer(lambda: _abi.check(L.byo_bfs_device(G.h, src, out.data_ptr(), None, pol,
                                                                                ctypes.byref(r)), ctx.h), 3)
            row["rounds"] = r.value
            row["bit_exact"] = bool(torch.equal(par, par2))
            tot["m20"] += row["ms_m20"]
            tot["learned"] += row["ms_learned"]
            g["bfs"].append(row)
        keys = torch.empty(2 * 1000000, dtype=torch.int64, device=dev)
        _abi.check(L.byo_gen_uniform_keys_device(ctx.h, 77, n, 1000000, keys.data_ptr()), ctx.h)

        def pair():
            _abi.check(L.byo_graph_insert_batch_device(G.h, keys.data_ptr(), keys.numel(), 0, ctypes.byref(ch)),
                       ctx.h)
            _abi.check(L.byo_graph_remove_batch_device(G.h, keys.data_ptr(), keys.numel(), 0, ctypes.byref(ch)),
                       ctx.h)
        for uname, up in (("merge", _abi.UPDATE_MERGE), ("learned_update", _abi.UPDATE_LEARNED)):
            _abi.check(L.byo_ctx_set_update_policy(ctx.h, up), ctx.h)
            pair()
            g["update_pair_ms_" + uname] = timer(pair, 3)
            tot[uname] += g["update_pair_ms_" + uname]
        _abi.check(L.byo_ctx_set_update_policy(ctx.h, _abi.UPDATE_MERGE), ctx.h)
        lab = torch.empty(n, dtype=torch.int32, device=dev)
        _abi.check(L.byo_cc_device(G.h, lab.data_ptr()), ctx.h)
        g["cc_ms"] = timer(lambda: _abi.check(L.byo_cc_device(G.h, lab.data_ptr()), ctx.h), 3)
        launches += ctx.launches - launches0
        comps[name] = g
        G.close()
        del par, par2, lab, keys
        torch.cuda.empty_cache()
    clk = clocks.stop()
    res = {"metric": "learned vs m/20 direction policy: summed BFS time over four graph families (bit-exact)",
           "value": tot["m20"] / tot["learned"], "unit": "speed-up of the learned policy (m20 time / learned time)",
           "n_gpus": world, "steps": 3, "warmup": 1, "ms_per_step": tot["learned"], "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u32 ids", "data": "synthetic (seeded graphs)",
           "config": {"workload": "C4 policy comparison (PMA container)"},
           "components": {"graphs": comps, "bfs_ms_total_m20": tot["m20"], "bfs_ms_total_learned": tot["learned"],
                          "update_ms_total_merge": tot["merge"],
                          "update_ms_total_learned": tot["learned_update"]},
           "gpu_launches": launches, "clocks": clk}
    return res, ctx, None


def mixed_cpu_sample(steps=None):
    """Bounded sample of the mixed stream on the oracle port: four of the
    query groups' sources as single-source BFS and two update batches."""
    from oracle import oracle as O
    O.build()
    s, d = O.rmat_edges(MIXED_SEED, MIXED_LG, MIXED_DRAWS)
    off, nb = O.build_csr(1 << MIXED_LG, s, d)
    del s, d
    deg = np.diff(off.astype(np.int64))
    qsrc = mixed_sources(deg.astype(np.uint32), MIXED_SEED)
    order, sizes = mixed_ops(MIXED_SEED)
    t0 = time.perf_counter()
    edges = 0.0
    nq = 4
    for s_ in qsrc[0][:nq]:
        par, _ = O.bfs(off, nb, int(s_))
        edges += deg[par != O.NONE].sum() / 2
    tq = time.perf_counter() - t0
    store = O.Store(off, nb)
    js = [int(np.argmin(sizes)), int(np.argmax(sizes))]
    keys_total = 0
    t1 = time.perf_counter()
    for j in js:
        us, ud = O.uniform_pairs(MIXED_SEED * 1000 + j, 1 << MIXED_LG, int(sizes[j]))
        k = O.keys_from_pairs(us, ud)
        store.insert_batch(k)
        store.remove_batch(k)
        keys_total += 2 * len(k)
    tu = time.perf_counter() - t1
    value = (edges + keys_total) / (tq + tu) / 1e9
    return {"value": value, "unit": MIXED_UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": "%d single-source BFS from the first query group's sources + insert/remove of batches "
                      "of %d and %d pairs on the oracle port (OpenMP, %d threads), %.1f s"
                      % (nq, sizes[js[0]], sizes[js[1]], O.num_threads(), tq + tu),
            "queries_per_s": nq / tq, "update_keys_per_s": keys_total / tu}


# ------------------------------------------------------------------ CPU (oracle) legs
_CPU_SETUP = {}


def cpu_setup(dynamic):
    if dynamic in _CPU_SETUP:
        return _CPU_SETUP[dynamic]
    _CPU_SETUP[dynamic] = _cpu_setup(dynamic)
    return _CPU_SETUP[dynamic]


def _cpu_setup(dynamic):
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
    """One step of the workload on the CPU restatement; returns (units, ms per
    phase, edges after the insert).  Phases: insert into the sorted-set store,
    export of its contents as the CSR the traversals read (the counterpart of
    the GPU container's compact snapshot, which the GPU arm rebuilds inside
    its BFS phase), BFS, CC, PageRank, remove."""
    t = [time.perf_counter()]
    if keys is not None:
        store.insert_batch(keys)
    t.append(time.perf_counter())
    if keys is not None:
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
    return float(units), np.diff(t) * 1e3, m


CPU_PHASES = ["insert", "export", "bfs", "cc", "pr", "remove"]


def run_reference(args, dynamic):
    O, off, nb, keys = cpu_setup(dynamic)
    store = O.Store(off, nb) if dynamic else None
    threads = O.num_threads()
    for _ in range(args.warmup):
        cpu_step(O, off, nb, keys, store)
    tot_units, tot_s = 0.0, 0.0
    ph_tot = np.zeros(len(CPU_PHASES))
    m_trav = len(nb)
    for _ in range(args.steps):
        u, ph, m_trav = cpu_step(O, off, nb, keys, store)
        tot_units += u
        tot_s += ph.sum() / 1e3
        ph_tot += ph
    value = tot_units / tot_s / 1e9
    sample = ("full steps of the workload on the oracle port (OpenMP), %d threads; each step's time includes "
              "the export of the store's contents as a CSR for the traversals (phase 'export', the counterpart "
              "of the GPU container's snapshot, which the GPU arm rebuilds inside its BFS phase)" % threads)
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_s * 1e3 / args.steps, "higher_is_better": True,
            "impl": "reference",
            "config": dynamic_config(dynamic, "pma", 1 << LG_N, m_trav),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample,
                             "phase_ms": {k: float(v) / args.steps for k, v in zip(CPU_PHASES, ph_tot)}},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "data": "synthetic (seeded RMAT, no dataset)"}


def cpu_baseline_sample(dynamic):
    O, off, nb, keys = cpu_setup(dynamic)
    store = O.Store(off, nb) if dynamic else None
    u, ph, _ = cpu_step(O, off, nb, keys, store)
    secs = ph.sum() / 1e3
    return {"value": u / secs / 1e9, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": "one full step of the same workload on the oracle port (OpenMP, %d threads), %.1f s, "
                      "including the export of the store as a CSR for the traversals" % (O.num_threads(), secs),
            "phase_ms": {k: float(v) for k, v in zip(CPU_PHASES, ph)}}


# ------------------------------------------------------------------ main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dynamic",
                    choices=["dynamic", "static", "mixed", "multi", "scale", "families", "map", "bytepd",
                             "stream", "tc"])
    ap.add_argument("--lg", type=int, default=0, help="multi: log2 vertices (default 24)")
    ap.add_argument("--container", default="pma", choices=["pma", "vos", "pcsr"],
                    help="dynamic: the container updated (pma: packed-memory array; vos: vector of per-vertex runs; "
                         "pcsr: packed CSR)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--policy", default="auto", choices=sorted(POLICIES) + ["auto"],
                    help="auto: the committed learned network if present, else m20")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="dynamic/static: skip the oracle check before timing")
    ap.add_argument("--no-sweep", action="store_true", help="dynamic: skip the 1e3/1e5/1e7 batch-size sweep")
    ap.add_argument("--no-pcsr", action="store_true", help="dynamic PMA: skip the same step on the packed CSR")
    ap.add_argument("--pr-launches", default="graph", choices=["graph", "stream"],
                    help="PageRank iterations as one CUDA graph (default) or one stream launch per kernel "
                         "(for per-kernel profiles)")
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
        if args.workload == "mixed":
            cb = mixed_cpu_sample()
            print(json.dumps({"metric": MIXED_METRIC, "value": cb["value"], "unit": MIXED_UNIT, "n_gpus": 0,
                              "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                              "impl": "reference", "config": {"workload": "mixed (bounded sample)"},
                              "cpu_baseline": cb, "data": "synthetic (seeded RMAT, uniform update pairs)",
                              "e2e": {"value": cb["value"], "unit": MIXED_UNIT, "h2d_bytes_per_step": 0,
                                      "d2h_bytes_per_step": 0}}), flush=True)
            return 0
        if args.workload in ("map", "bytepd", "tc"):
            cb = {"map": map_cpu_sample, "bytepd": bytepd_cpu_sample, "tc": tc_cpu_sample}[args.workload]()
            metric = {"map": "Test_Map + Test_Map_Remote edges/s (run_all's Map applications)",
                      "bytepd": "byte-PD decode edges/s (compressed neighbour lists to CSR on the GPU)",
                      "tc": "TriangleCounting (degree-ordered) edges/s on RMAT 2^22, average degree 32"}[args.workload]
            print(json.dumps({"metric": metric,
                              "value": cb["value"], "unit": cb["unit"], "n_gpus": 0, "steps": args.steps,
                              "warmup": args.warmup, "higher_is_better": True, "impl": "reference",
                              "config": {"workload": args.workload + " (bounded sample)"}, "cpu_baseline": cb,
                              "data": "synthetic (seeded RMAT)",
                              "e2e": {"value": cb["value"], "unit": cb["unit"], "h2d_bytes_per_step": 0,
                                      "d2h_bytes_per_step": 0}}), flush=True)
            return 0
        print(json.dumps(run_reference(args, dynamic)), flush=True)
        return 0

    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    if args.workload == "mixed":
        res, ctx, G = run_mixed(args, rank, world, local_rank)
    elif args.workload == "multi":
        res, ctx, G = run_multi(args, rank, world, local_rank)
        args.no_cpu_baseline = True
    elif args.workload == "map":
        res, ctx, G = run_map(args, rank, world, local_rank)
        if rank == 0 and not args.no_cpu_baseline:
            res["cpu_baseline"] = map_cpu_sample()
        args.no_cpu_baseline = True
    elif args.workload == "stream":
        res, ctx, G = run_stream(args, rank, world, local_rank)
        args.no_cpu_baseline = True
    elif args.workload == "tc":
        res, ctx, G = run_tc(args, rank, world, local_rank)
        if rank == 0 and not args.no_cpu_baseline:
            res["cpu_baseline"] = tc_cpu_sample()
        args.no_cpu_baseline = True
    elif args.workload == "bytepd":
        res, ctx, G = run_bytepd(args, rank, world, local_rank)
        if rank == 0 and not args.no_cpu_baseline:
            res["cpu_baseline"] = bytepd_cpu_sample()
        args.no_cpu_baseline = True
    elif args.workload in ("scale", "families"):
        fn = run_scale if args.workload == "scale" else run_families
        res, ctx, G = fn(args, rank, world, local_rank)
        args.no_cpu_baseline = True
    else:
        res, ctx, G = run_ours(args, rank, world, local_rank)
    if G is not None:
        G.close()
    ctx.close()
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            res["cpu_baseline"] = mixed_cpu_sample() if args.workload == "mixed" else cpu_baseline_sample(dynamic)
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
