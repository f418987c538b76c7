"""NumPy reference of the learned preconditioner's message-passing network, in
float64 with the weights rounded to BF16 as the CUDA kernels read them: forward
pass, loss and gradients, for checking dgc_mpnn_train_step / dgc_mpnn_forward.

Parameter layout (flat, as dgc_mpnn_get_weights returns it), W = 64:
  Win [W][npi], bin [W], then per layer Ws [W][W], Wn [W][W], b [W],
  then Wout [npi][W], bout [npi].
"""
import numpy as np

W = 64


def bf16_round(x):
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w, npi, L):
    w = bf16_round(w)
    o = 0
    P = {}
    P["Win"] = w[o:o + W * npi].reshape(W, npi); o += W * npi
    P["bin"] = w[o:o + W]; o += W
    P["Ws"], P["Wn"], P["b"] = [], [], []
    for _ in range(L):
        P["Ws"].append(w[o:o + W * W].reshape(W, W)); o += W * W
        P["Wn"].append(w[o:o + W * W].reshape(W, W)); o += W * W
        P["b"].append(w[o:o + W]); o += W
    P["Wout"] = w[o:o + npi * W].reshape(npi, W); o += npi * W
    P["bout"] = w[o:o + npi]; o += npi
    assert o == w.size
    return P


def neighbour_sum(h, nbr, K):
    """m[e] = sum of h over the face neighbours (nbr: K x 4 codes, cell << 2 | face or < 0)."""
    S = h.shape[0] // K
    m = np.zeros_like(h)
    for s in range(S):
        hs = h[s * K:(s + 1) * K]
        ms = m[s * K:(s + 1) * K]
        for f in range(3):
            c = nbr[:, f]
            ok = c >= 0
            ms[ok] += hs[c[ok] >> 2]
    return m


def forward(w, x, nbr, K, npi, L, linear=False):
    """x: (S*K, npi) -> y (S*K, npi) and the activations (linear: no ReLU)."""
    P = unpack(w, npi, L)
    hs = [x @ P["Win"].T + P["bin"]]
    acts = []
    for l in range(L):
        h = hs[-1]
        m = neighbour_sum(h, nbr, K)
        a = h @ P["Ws"][l].T + m @ P["Wn"][l].T + P["b"][l]
        acts.append(a)
        hs.append(h + (a if linear else np.maximum(a, 0.0)))
    y = hs[-1] @ P["Wout"].T + P["bout"]
    return y, hs, acts, P


def loss_and_grad(w, x, t, nbr, K, npi, np_valid, L, spd=None, linear=False):
    """Loss = mean over samples of |y - t|^2 / |t|^2 on valid nodes, or with
    spd (a symmetric operator on one (K, npi) field, padding zero) the energy
    form d.S d / t.S t; returns (loss, flat gradient).  linear: the network
    without ReLU, whose bias gradients are zero (the biases are held at zero)."""
    S = x.shape[0] // K
    y, hs, acts, P = forward(w, x, nbr, K, npi, L, linear)
    mask = np.zeros(npi)
    mask[:np_valid] = 1.0
    dy = np.zeros_like(y)
    loss = 0.0
    for s in range(S):
        sl = slice(s * K, (s + 1) * K)
        d = (y[sl] - t[sl]) * mask
        tm = t[sl] * mask
        if spd is None:
            tn = np.sum(tm * tm)
            loss += np.sum(d * d) / tn / S
            dy[sl] = 2.0 * d / tn / S
        else:
            Sd = spd(d) * mask
            tn = np.sum(tm * (spd(tm) * mask))
            loss += np.sum(d * Sd) / tn / S
            dy[sl] = 2.0 * Sd / tn / S
    g = {"Wout": dy.T @ hs[-1], "bout": dy.sum(0)}
    dh = dy @ P["Wout"]
    gWs, gWn, gb = [None] * L, [None] * L, [None] * L
    for l in range(L - 1, -1, -1):
        h = hs[l]
        gg = dh if linear else dh * (acts[l] > 0.0)
        m = neighbour_sum(h, nbr, K)
        gWs[l] = gg.T @ h
        gWn[l] = gg.T @ m
        gb[l] = gg.sum(0)
        dh = dh + gg @ P["Ws"][l] + neighbour_sum(gg, nbr, K) @ P["Wn"][l]
    g["Win"] = dh.T @ x
    g["bin"] = dh.sum(0)
    flat = [g["Win"].ravel(), g["bin"]]
    for l in range(L):
        flat += [gWs[l].ravel(), gWn[l].ravel(), gb[l]]
    flat += [g["Wout"].ravel(), g["bout"]]
    if linear:  # bin, the per-layer b and bout
        for i in [1] + [4 + 3 * l for l in range(L)] + [len(flat) - 1]:
            flat[i] = np.zeros_like(flat[i])
    return loss, np.concatenate(flat)
