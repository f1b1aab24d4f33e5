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
it, and the m/20 rule stays the fallback and the judge inside the engine.
"""
import ctypes

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


JUDGE_MARGIN = 0.05  # the engine's kJudgeMargin


def round_choices(ctx, params, X, fallback):
    """The engine's decision rule applied to predictions: argmin over the
    three directions unless the rule's choice is within the judge margin."""
    P = forward(ctx, params, X)[:, :3]
    best = P.argmin(1)
    keep = P[np.arange(len(P)), fallback] - P[np.arange(len(P)), best] <= JUDGE_MARGIN
    return np.where(keep, fallback, best)


def round_cost(Y, choice):
    """Total microseconds of the rounds under a choice per round."""
    return float(micros(Y[np.arange(len(Y)), choice]).sum())
