"""The learned direction / update policy: sample collection from the engine's
own logs, training on the device, evaluation against the m/20 rule.

Round samples come from BFS runs with every round timed: for each source the
traversal is run with push, pull and blocked forced every round.  The
frontier of round r is the same in all three runs (BFS levels do not depend on
the direction), so each round yields one sample: its features and the three
times.  A run under the m/20 rule (edge_map_data.h:254-307) records the rule's
choice for the same rounds.  Update samples time a batch as in-place merge and
as rebuild (byo_update_sample).

Targets are log2(1 + microseconds) / 16.  A trained network is installed with
install(); BFS(..., policy=POLICY_LEARNED) and update policy UPDATE_LEARNED use
it, and the m/20 rule stays the fallback and the arbiter inside the engine.
"""
import argparse
import ctypes
import json
import os
import time

import numpy as np

from . import _abi
from ._abi import check, lib

NF, NO, NP = _abi.POLICY_NFEATURES, _abi.POLICY_NOUTPUTS, _abi.POLICY_NPARAMS
MODES = (_abi.POLICY_PUSH, _abi.POLICY_PULL, _abi.POLICY_BLOCKED)  # outputs 0, 1, 2


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def target(ms):
    return np.log2(1.0 + np.asarray(ms, np.float64) * 1000.0) / 16.0


def micros(t):
    return np.exp2(np.asarray(t, np.float64) * 16.0) - 1.0


def collect_round_samples(G, sources, warm=True):
    """Returns X[n,16], Y[n,5], mask[n], m20_choice[n] (0 push, 1 pull)."""
    from .graph import BFS
    ctx = G.ctx
    X, Y, M, C = [], [], [], []
    ctx.set_round_timing(True)
    try:
        for s in sources:
            if warm:
                BFS(G, s, policy=_abi.POLICY_M20)
            logs = {}
            for mode in MODES + (_abi.POLICY_M20,):
                BFS(G, s, policy=mode)
                logs[mode] = ctx.last_rounds()
            nr = min(len(v) for v in logs.values())
            for r in range(nr):
                X.append(logs[_abi.POLICY_PUSH][r]["features"])
                Y.append([target(logs[m][r]["ms"]) for m in MODES] + [0.0, 0.0])
                M.append(0b00111)
                C.append(logs[_abi.POLICY_M20][r]["mode"])
    finally:
        ctx.set_round_timing(False)
    return (np.array(X, np.float32).reshape(-1, NF), np.array(Y, np.float32).reshape(-1, NO),
            np.array(M, np.uint8), np.array(C, np.int64))


def collect_update_samples(G, batches):
    X, Y, M = [], [], []
    for keys in batches:
        k = np.ascontiguousarray(keys, np.uint64)
        x = np.zeros((2, NF), np.float32)
        y = np.zeros((2, NO), np.float32)
        m = np.zeros(2, np.uint8)
        check(lib().byo_update_sample(G.h, _ptr(k), len(k), _ptr(x), _ptr(y), _ptr(m)), G.ctx.h)
        X.append(x)
        Y.append(y)
        M.append(m)
    return np.concatenate(X), np.concatenate(Y), np.concatenate(M)


def init_params(seed=1):
    p = np.zeros(NP, np.float32)
    check(lib().byo_policy_init_params(seed, _ptr(p)))
    return p


def train(ctx, X, Y, M, epochs=400, lr=3e-3, seed=1, init=None):
    """Trains on the device; installs and returns (params, loss per epoch)."""
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    M = np.ascontiguousarray(M, np.uint8)
    losses = np.zeros(epochs, np.float32)
    ip = None if init is None else _ptr(np.ascontiguousarray(init, np.float32))
    check(lib().byo_policy_train(ctx.h, ip, _ptr(X), _ptr(Y), _ptr(M), len(X), epochs, lr, seed, _ptr(losses)),
          ctx.h)
    return get_params(ctx), losses


def get_params(ctx):
    p = np.zeros(NP, np.float32)
    check(lib().byo_policy_get_params(ctx.h, _ptr(p)), ctx.h)
    return p


def install(ctx, params):
    p = np.ascontiguousarray(params, np.float32)
    assert p.size == NP
    check(lib().byo_policy_set_params(ctx.h, _ptr(p)), ctx.h)


def clear(ctx):
    check(lib().byo_policy_clear(ctx.h), ctx.h)


def forward(ctx, params, X):
    X = np.ascontiguousarray(X, np.float32).reshape(-1, NF)
    Y = np.zeros((len(X), NO), np.float32)
    check(lib().byo_policy_forward(ctx.h, _ptr(np.ascontiguousarray(params, np.float32)), _ptr(X), len(X),
                                   _ptr(Y)), ctx.h)
    return Y


def loss_grad(ctx, params, X, Y, M):
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    M = np.ascontiguousarray(M, np.uint8)
    g = np.zeros(NP, np.float32)
    loss = ctypes.c_float(0)
    check(lib().byo_policy_loss_grad(ctx.h, _ptr(np.ascontiguousarray(params, np.float32)), _ptr(X), _ptr(Y),
                                     _ptr(M), len(X), ctypes.byref(loss), _ptr(g)), ctx.h)
    return float(loss.value), g


ARBITER_MARGIN = 0.006  # the engine's kArbiterMargin (a predicted gain of about 7%)
GATE_FACTOR = 64      # the engine's kGateFactor
GATE_HUB_BIN = 5      # the engine's kGateHubBin (degree >= 4^5)


def round_choices(ctx, params, X, fallback):
    """The engine's decision rule applied to predictions: argmin over the
    three directions unless the rule's choice is within the arbiter margin, and
    the rule alone for frontiers far below its threshold without a hub
    (feature 14 is (|F| + outdeg) / (m/20), features 6..13 the degree
    histogram by powers of 4)."""
    P = forward(ctx, params, X)[:, :3]
    best = P.argmin(1)
    keep = P[np.arange(len(P)), fallback] - P[np.arange(len(P)), best] <= ARBITER_MARGIN
    hub = (X[:, 6 + GATE_HUB_BIN:14] > 0).any(1)
    keep |= (X[:, 14] * GATE_FACTOR <= 1.0) & ~hub
    return np.where(keep, fallback, best)


def round_cost(Y, choice):
    """Total microseconds of the rounds under a choice per round."""
    return float(micros(Y[np.arange(len(Y)), choice]).sum())


# ------------------------------------------------------------------ training run
DEFAULT_PARAMS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "policy_gb300.npy")


def load_default(ctx, path=DEFAULT_PARAMS):
    """Installs the committed network if present; returns True if it did."""
    if not os.path.exists(path):
        return False
    install(ctx, np.load(path))
    return True


def _graphs(ctx, scale):
    """Training graphs of 2^(18 + scale) vertices (seeds unlike the benchmark
    graphs'): RMAT dense and sparse, ER, a square grid, Chung-Lu."""
    from .graph import Graph
    s = scale
    yield "rmat", Graph.generate(ctx, "rmat", seed=101 + s, lg_n=18 + s, draws=1 << (22 + s))
    yield "rmat-sparse", Graph.generate(ctx, "rmat", seed=102 + s, lg_n=18 + s, draws=1 << (20 + s))
    yield "er", Graph.generate(ctx, "er", seed=103 + s, n=1 << (18 + s), draws=1 << (21 + s))
    yield "grid", Graph.generate(ctx, "grid", n=1 << (8 + s // 2), draws=1 << (8 + s // 2))
    yield "chung-lu", Graph.generate(ctx, "chung_lu", seed=104 + s, n=1 << (18 + s), draws=1 << (21 + s),
                                     exponent=2.1)


def main():
    ap = argparse.ArgumentParser(description="collect engine timings on this GPU and train the policy")
    ap.add_argument("--out", default=DEFAULT_PARAMS)
    ap.add_argument("--scales", default="0,2,4,6", help="graphs of 2^(18+scale) vertices, for each scale")
    ap.add_argument("--large", type=int, default=8, help="also RMAT graphs of 2^(18+large) vertices (0: none)")
    ap.add_argument("--sources", type=int, default=12)
    ap.add_argument("--epochs", type=int, default=600)
    args = ap.parse_args()
    from .graph import Context, Graph
    ctx = Context(0)
    t0 = time.time()
    tr, te, report = [], [], {}
    def graphs():
        for sc in [int(x) for x in args.scales.split(",") if x]:
            for name, G in _graphs(ctx, sc):
                yield "%s-%d" % (name, 18 + sc), G
        if args.large:
            lg = 18 + args.large
            for name, draws in (("rmat", 1 << (lg + 4)), ("rmat-sparse", 1 << (lg + 2))):
                yield "%s-%d" % (name, lg), Graph.generate(ctx, "rmat", seed=111 + len(name), lg_n=lg, draws=draws)
            yield "er-%d" % lg, Graph.generate(ctx, "er", seed=113, n=1 << lg, draws=1 << (lg + 4))

    for name, G in graphs():
        deg = G.degrees()
        rng = np.random.default_rng(G.N() + len(name))
        srcs = rng.choice(np.nonzero(deg)[0], args.sources, replace=False)
        k = (2 * args.sources) // 3
        tr.append(collect_round_samples(G, srcs[:k]))
        te.append((name, collect_round_samples(G, srcs[k:], warm=False)))
        G.close()
        print(name, "samples", len(tr[-1][0]), "%.1fs" % (time.time() - t0), flush=True)
    # update samples on the packed-memory-array container: symmetrised uniform
    # batches, log-uniform sizes
    uxs, uys, ums = [], [], []
    for lg in (20, 22, 24, 18 + args.large if args.large else 24):
        G = Graph.generate(ctx, "rmat", seed=105 + lg, lg_n=lg, draws=1 << (lg + 4), container="pma")
        n = G.N()
        rng = np.random.default_rng(lg)
        batches = []
        for b in np.unique(np.logspace(2, 7, 11).astype(np.int64)):
            u = rng.integers(0, n, b, dtype=np.uint64)
            v = rng.integers(0, n, b, dtype=np.uint64)
            batches.append(np.concatenate([(u << np.uint64(32)) | v, (v << np.uint64(32)) | u]))
        x, y, mk = collect_update_samples(G, batches)
        uxs.append(x)
        uys.append(y)
        ums.append(mk)
        G.close()
        print("updates lg", lg, "%.1fs" % (time.time() - t0), flush=True)
    ux, uy, um = np.concatenate(uxs), np.concatenate(uys), np.concatenate(ums)
    X = np.concatenate([t[0] for t in tr] + [ux])
    Y = np.concatenate([t[1] for t in tr] + [uy])
    M = np.concatenate([t[2] for t in tr] + [um])
    params, losses = train(ctx, X, Y, M, epochs=args.epochs, lr=3e-3, seed=1)
    for name, (Xt, Yt, Mt, Ct) in te:
        ch = round_choices(ctx, params, Xt, Ct)
        report[name] = {"rounds": int(len(Xt)), "m20_us": round_cost(Yt, Ct), "learned_us": round_cost(Yt, ch),
                        "best_us": round_cost(Yt, Yt[:, :3].argmin(1))}
    pu = forward(ctx, params, ux)
    upd = {"samples": int(len(ux)), "merge_us": float(micros(uy[:, 3]).sum()),
           "learned_us": float(micros(np.where(pu[:, 3] - pu[:, 4] > ARBITER_MARGIN, uy[:, 4], uy[:, 3])).sum()),
           "best_us": float(micros(uy[:, 3:5].min(1)).sum())}
    np.save(args.out, params)
    meta = {"train_samples": int(len(X)), "epochs": args.epochs, "loss_first": float(losses[0]),
            "loss_last": float(losses[-1]), "held_out_rounds": report, "updates_in_sample": upd,
            "seconds": round(time.time() - t0, 1)}
    with open(os.path.splitext(args.out)[0] + ".json", "w") as f:
        json.dump(meta, f, indent=1)
    print(json.dumps(meta))
    ctx.close()


if __name__ == "__main__":
    main()
