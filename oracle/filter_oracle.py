"""CPU oracle of the learned candidate filter -- TEST INFRASTRUCTURE ONLY.

Only tests/ (and the CPU-baseline leg of bench.py) may import this module; the product
path never does.  It restates, in numpy, what canu_gb300/csrc/oic_filter.cu computes:

  features(...)   the 80-value FP16 feature row of one candidate pair from its match
                  runs (the Match_Node_t lists of overlapInCore-Find_Overlaps.C:25-96:
                  T offset, run length, S start; a run of length L holds L-K+1 seeds)
  forward(...)    the 80 -> 128 -> 128 -> 1 network with FP16 parameters, FP16
                  activations after bias + ReLU, and float64 accumulation (the kernels
                  accumulate in FP32; tests compare with a tolerance)
  backward(...)   the gradient of sum_i w_i * BCE(sigmoid(z_i), y_i) with the same FP16
                  rounding points as the kernels (dz2, dz1 rounded to FP16)
  numeric_grad()  central differences of the unrounded float64 network, to pin
                  backward() itself

The filter has no counterpart in the reference (overlapInCore extends every candidate
pair, overlapInCore-Process_String_Overlaps.C:354-547); its labels come from the exact
path, which is pinned against the reference separately.
"""
import numpy as np

IN, HID = 80, 128
OFF = {"w1": (0, (HID, IN)), "b1": (10240, (HID,)), "w2": (10368, (HID, HID)),
       "b2": (26752, (HID,)), "w3": (26880, (HID,)), "b3": (27008, (1,))}
NPARAM = 27009


def unpack(params):
    """Parameter array (float16 or float64, NPARAM) -> dict of float64 arrays."""
    p = np.asarray(params).astype(np.float64)
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in OFF.items()}


def pack(d, dtype=np.float64):
    out = np.zeros(NPARAM, dtype=dtype)
    for k, (o, s) in OFF.items():
        out[o:o + int(np.prod(s))] = np.asarray(d[k]).reshape(-1)
    return out


def init_params(seed=0):
    """He-uniform weights, zero biases; input columns 67..79 stay zero."""
    r = np.random.default_rng(seed)
    d = {k: np.zeros(s) for k, (o, s) in OFF.items()}
    d["w1"][:, :67] = r.uniform(-1, 1, (HID, 67)) * np.sqrt(6.0 / 67)
    d["w2"][:] = r.uniform(-1, 1, (HID, HID)) * np.sqrt(6.0 / HID)
    d["w3"][:] = r.uniform(-1, 1, HID) * np.sqrt(3.0 / HID)
    return pack(d).astype(np.float16)


def features(len_s, len_t, seeds, runs, k):
    """Feature row (float16[80]) of one pair; runs = iterable of (tOff, len, sOff)."""
    span = int(len_s) + int(len_t)
    hist = np.zeros(64, dtype=np.int64)
    for t_off, ln, s_off in np.asarray(runs, dtype=np.int64).reshape(-1, 3):
        b = ((t_off - s_off + len_s) * 64) // span
        hist[min(max(b, 0), 63)] += ln - k + 1
    row = np.zeros(IN, dtype=np.float32)
    for b in range(64):
        dc = ((2 * b + 1) * span) // 128 - len_s            # centre diagonal of the bin
        ol = min(len_s, len_t - dc) - (-dc if dc < 0 else 0)
        ol = max(ol, 64)
        v = np.float32(hist[b]) / np.float32(ol)
        row[b] = min(v, np.float32(4.0))
    row[64] = (np.log(np.float32(len_s)) - np.float32(8)) * np.float32(0.5)
    row[65] = (np.log(np.float32(len_t)) - np.float32(8)) * np.float32(0.5)
    row[66] = (np.log(np.float32(1) + np.float32(seeds)) - np.float32(5)) * np.float32(0.25)
    return row.astype(np.float16)


def _f16(a):
    return np.asarray(a).astype(np.float16).astype(np.float64)


def forward(params, x, round_act=True):
    """(logit[n], h1[n,128], h2[n,128]); x = float16 [n, 80]."""
    P = unpack(params)
    X = np.asarray(x).astype(np.float64)
    rnd = _f16 if round_act else (lambda a: a)
    h1 = rnd(np.maximum(X @ P["w1"].T + P["b1"], 0.0))
    h2 = rnd(np.maximum(h1 @ P["w2"].T + P["b2"], 0.0))
    return h2 @ P["w3"] + P["b3"][0], h1, h2


def loss(params, x, y, w, round_act=False):
    z, _, _ = forward(params, x, round_act)
    return float(np.sum(w * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))))


def backward(params, x, h1, h2, logit, y, w, round_grad=True):
    """Gradient (float64[NPARAM]) and loss, the kernels' rounding points."""
    P = unpack(params)
    X = np.asarray(x).astype(np.float64)
    z = np.asarray(logit, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    w = np.ones_like(z) if w is None else np.asarray(w, dtype=np.float64)
    rnd = _f16 if round_grad else (lambda a: a)
    p = 1.0 / (1.0 + np.exp(-z))
    dl = w * (p - y)
    lsum = float(np.sum(w * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))))
    dz2 = rnd(dl[:, None] * P["w3"][None, :] * (h2 > 0))
    dz1 = rnd((dz2 @ P["w2"]) * (h1 > 0))
    g = {"w1": dz1.T @ X, "b1": dz1.sum(0), "w2": dz2.T @ h1, "b2": dz2.sum(0), "w3": dl @ h2,
         "b3": np.array([dl.sum()])}
    return pack(g), lsum


def numeric_grad(params, x, y, w, idx, eps=1e-5):
    """Central differences of the unrounded float64 loss at parameter indices idx."""
    base = np.asarray(params, dtype=np.float64)
    out = []
    for i in idx:
        a, b = base.copy(), base.copy()
        a[i] += eps
        b[i] -= eps
        out.append((loss(a, x, y, w) - loss(b, x, y, w)) / (2 * eps))
    return np.array(out)
