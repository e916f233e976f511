"""CPU oracle of the learner's sketch and selectivity network -- test
infrastructure only.

The reference evaluator has no learned component, so this oracle is not a
restatement of reference code: it is the mathematical definition the GPU
kernels implement, in float64 numpy, used to check their forward pass, loss and
gradients.  It is itself checked against central finite differences
(tests/test_learned.py), which pins it without any reference artefact.

Network: x[F] -> ReLU(W1 x + b1)[H] -> ReLU(W2 h1 + b2)[H] -> z = W3 h2 + b3 [O].
Prediction of conjunct o's selectivity: sigmoid(z_o); its log is
-softplus(-z_o).  Loss over M examples: mean over M*O of (log sigmoid(z) - y)^2,
y = log(measured pass fraction + 1e-6).
Flat parameter layout: W1[H*F] b1[H] W2[H*H] b2[H] W3[O*H] b3[O], row-major
(out x in).
"""
from __future__ import annotations

import numpy as np


def param_count(F: int, H: int, O: int) -> int:
    return H * F + H + H * H + H + O * H + O


def unpack(p: np.ndarray, F: int, H: int, O: int):
    p = np.asarray(p, dtype=np.float64)
    o = 0

    def take(k, shape):
        nonlocal o
        v = p[o:o + k].reshape(shape)
        o += k
        return v

    W1 = take(H * F, (H, F))
    b1 = take(H, (H,))
    W2 = take(H * H, (H, H))
    b2 = take(H, (H,))
    W3 = take(O * H, (O, H))
    b3 = take(O, (O,))
    return W1, b1, W2, b2, W3, b3


def softplus(x: np.ndarray) -> np.ndarray:
    return np.maximum(x, 0.0) + np.log1p(np.exp(-np.abs(x)))


def forward(p, X, F: int, H: int, O: int):
    W1, b1, W2, b2, W3, b3 = unpack(p, F, H, O)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    z = h2 @ W3.T + b3
    return h1, h2, z


def loss(p, X, Y, F: int, H: int, O: int) -> float:
    _, _, z = forward(p, X, F, H, O)
    d = -softplus(-z) - np.asarray(Y, dtype=np.float64)
    return float(np.mean(d * d))


def grad(p, X, Y, F: int, H: int, O: int):
    """(gradient in the flat layout, loss, z)."""
    W1, b1, W2, b2, W3, b3 = unpack(p, F, H, O)
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    h1, h2, z = forward(p, X, F, H, O)
    M = X.shape[0]
    ls = -softplus(-z)
    d = ls - Y
    L = float(np.mean(d * d))
    dz = 2.0 / (M * O) * d * (1.0 / (1.0 + np.exp(z)))   # d log sigmoid(z)/dz = sigmoid(-z)
    gW3 = dz.T @ h2
    gb3 = dz.sum(axis=0)
    dh2 = (dz @ W3) * (h2 > 0)
    gW2 = dh2.T @ h1
    gb2 = dh2.sum(axis=0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    gW1 = dh1.T @ X
    gb1 = dh1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return g, L, z


def finite_difference(p, X, Y, F: int, H: int, O: int, idx, eps: float = 1e-6) -> np.ndarray:
    """Central differences of the loss at parameter indices idx."""
    p = np.asarray(p, dtype=np.float64).copy()
    out = []
    for i in idx:
        old = p[i]
        p[i] = old + eps
        lp = loss(p, X, Y, F, H, O)
        p[i] = old - eps
        lm = loss(p, X, Y, F, H, O)
        p[i] = old
        out.append((lp - lm) / (2 * eps))
    return np.array(out)


def sketch_features(values, valid, anchors, stride_words: int = 64) -> np.ndarray:
    """The learner's per-batch sketch (11 features per column) of the rows in
    every stride_words-th 32-row word: min and max of t / 16, cumulative
    fractions of the 8 bins of t (t < -8, [-8, -4), [-4, -1), [-1, 0), t == 0,
    (0, 1], (1, 4], t > 4) and the null fraction, with t = sign(d) log1p(|d|),
    d = value - anchor computed in float64 then rounded to float32.
    values: list of numpy arrays; valid: list of bool arrays or None."""
    out = []
    for j, x in enumerate(values):
        n = len(x)
        nw = (n + 31) // 32
        idx = (np.arange(0, nw, stride_words)[:, None] * 32 + np.arange(32)[None, :]).ravel()
        idx = idx[idx < n]
        ok = np.ones(len(idx), dtype=bool) if valid[j] is None else valid[j][idx]
        d = (x[idx][ok].astype(np.float64) - anchors[j]).astype(np.float32)
        t = (np.sign(d) * np.log1p(np.abs(d).astype(np.float64))).astype(np.float32)
        nv = len(t)
        if nv == 0:
            out += [0.0] * 10
        else:
            h = np.array([(t < -8).sum(), ((t >= -8) & (t < -4)).sum(), ((t >= -4) & (t < -1)).sum(),
                          ((t >= -1) & (t < 0)).sum(), (t == 0).sum(), ((t > 0) & (t <= 1)).sum(),
                          ((t > 1) & (t <= 4)).sum(), (t > 4).sum()], dtype=np.float64)
            out += [float(t.min()) / 16, float(t.max()) / 16] + list(np.cumsum(h) / nv)
        out.append((len(idx) - nv) / len(idx) if len(idx) else 0.0)
    return np.array(out, dtype=np.float64)


def word_loads(columns_by_conjunct, keep_by_conjunct, order) -> int:
    """32-row words each conjunct reads when evaluated in `order` with per-word
    short-circuit: a conjunct is evaluated for a word while any row of the word
    is still alive.  keep_by_conjunct[c] is the boolean pass vector of conjunct
    c over the batch."""
    n = len(keep_by_conjunct[0])
    nwords = (n + 31) // 32
    pad = nwords * 32 - n
    alive = np.ones(n, dtype=bool)
    loads = 0
    for c in order:
        words_alive = np.pad(alive, (0, pad)).reshape(nwords, 32).any(axis=1)
        loads += int(words_alive.sum()) * columns_by_conjunct[c]
        alive &= keep_by_conjunct[c]
    return loads
