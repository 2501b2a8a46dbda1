"""FP32 NumPy restatement of the move-ordering network (test oracle only):
features, forward pass, softmax cross-entropy over the legal moves and the
full backward pass, for the gradient check of the tensor-core kernels."""
from __future__ import annotations

import numpy as np

import oracle_lib as ol

SHAPES = [("W1", (512, 768)), ("b1", (512,)), ("W2", (256, 512)), ("b2", (256,)), ("W3", (128, 256)),
          ("b3", (128,)), ("Ef", (64, 64)), ("Et", (64, 64))]


def unflatten(p):
    out, off = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = p[off:off + n].reshape(shape).astype(np.float32)
        off += n
    return out


def flatten(d):
    return np.concatenate([d[name].reshape(-1) for name, _ in SHAPES]).astype(np.float32)


def features(board, stm):
    """768 one-hot inputs from the side to move; legal moves as (from, to)
    in the same (mirrored) frame; the move list in oracle order."""
    x = np.zeros(768, dtype=np.float32)
    flip = 56 if stm else 0
    occ = int(board[1]) | int(board[2]) | int(board[3])
    for sq in range(64):
        if not (occ >> sq) & 1:
            continue
        pc = ((int(board[0]) >> sq) & 1) | (((int(board[1]) >> sq) & 1) << 1) | \
             (((int(board[2]) >> sq) & 1) << 2) | (((int(board[3]) >> sq) & 1) << 3)
        plane = (6 if (pc & 1) != stm else 0) + (pc >> 1) - 1
        x[plane * 64 + (sq ^ flip)] = 1.0
    moves = ol.genmoves(board, stm)
    ft = [((m & 63) ^ flip, ((m >> 6) & 63) ^ flip) for m in moves]
    return x, moves, ft


def loss_and_grads(p, boards, stm, targets, bf16_weights=True):
    P = unflatten(p)
    if bf16_weights:  # the kernels multiply with BF16 copies of the weights
        for k in ("W1", "W2", "W3"):
            P[k] = to_bf16(P[k])
    n = len(stm)
    X, lists = [], []
    for i in range(n):
        x, moves, ft = features(boards[i], int(stm[i]))
        X.append(x)
        t = moves.index(int(targets[i])) if int(targets[i]) in moves else -1
        lists.append((ft, t))
    X = np.stack(X)
    H1 = np.maximum(X @ P["W1"].T + P["b1"], 0)
    H2 = np.maximum(H1 @ P["W2"].T + P["b2"], 0)
    Q = H2 @ P["W3"].T + P["b3"]
    G = {k: np.zeros_like(v) for k, v in P.items()}
    dQ = np.zeros_like(Q)
    loss = 0.0
    for i, (ft, t) in enumerate(lists):
        if t < 0 or not ft:
            continue
        f = np.array([a for a, _ in ft])
        to = np.array([b for _, b in ft])
        qf, qt = Q[i, :64], Q[i, 64:]
        logit = P["Ef"][f] @ qf + P["Et"][to] @ qt
        mx = logit.max()
        e = np.exp(logit - mx)
        pr = e / e.sum()
        loss += (mx + np.log(e.sum())) - logit[t]
        dl = pr.copy()
        dl[t] -= 1.0
        dl /= n
        dQ[i, :64] = dl @ P["Ef"][f]
        dQ[i, 64:] = dl @ P["Et"][to]
        np.add.at(G["Ef"], f, np.outer(dl, qf))
        np.add.at(G["Et"], to, np.outer(dl, qt))
    dH2 = (dQ @ P["W3"]) * (H2 > 0)
    G["W3"] = dQ.T @ H2
    G["b3"] = dQ.sum(0)
    dH1 = (dH2 @ P["W2"]) * (H1 > 0)
    G["W2"] = dH2.T @ H1
    G["b2"] = dH2.sum(0)
    G["W1"] = dH1.T @ X
    G["b1"] = dH1.sum(0)
    return loss / n, G


def to_bf16(a):
    """round-to-nearest-even to bfloat16, returned as float32"""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)
