"""Training and evaluation of the learned candidate filter.

    python -m canu_gb300.filter_train --workload c2 --train-seeds 1,2,3,4,5 --eval-seed 6 \\
        --out canu_gb300/filter_c2.npz

1. Labels: for each training seed the workload's reads are generated and run through
   the exact GPU path with pair collection on; a candidate pair is positive when the
   DP emitted an overlap record for it.  Its feature row comes from the same run.
2. Training: the network (80 -> 128 -> 128 -> 1, FP16 parameters) is trained on the
   GPU by the library's own kernels -- oic_mlp_forward, oic_mlp_backward (FP16
   tensor-core GEMMs, FP32 accumulation) and oic_mlp_adam (FP32 master weights).
   PyTorch only holds the device buffers and draws the minibatch permutation.
3. Threshold: the largest score cut that keeps `recall` of the training positives.
4. Evaluation on the held-out seed: a plain run and a filtered run of the same reads;
   recall is |filtered records ∩ plain records| / |plain records| on (a_iid, b_iid,
   flipped), and every filtered record must equal its plain record word for word.

Negative pairs are weighted by the DP work they cost (pairs that end before the DP
cost nothing to keep), positives by a fixed factor, so the loss spends its capacity
where the filter saves time.
"""
import argparse
import json
import math
import os
import time

import numpy as np

from . import (FILTER_IN, FILTER_NPARAM, Overlapper, mlp_adam, mlp_backward, mlp_forward, sort_records,
               workloads)

# FP16 parameter layout (include/oic_gpu.h)
_OFF = {"w1": (0, (128, 80)), "b1": (10240, (128,)), "w2": (10368, (128, 128)), "b2": (26752, (128,)),
        "w3": (26880, (128,)), "b3": (27008, (1,))}


def init_params(seed=0):
    """He-uniform weights and zero biases; the 13 padding inputs keep zero weights."""
    r = np.random.default_rng(seed)
    p = np.zeros(FILTER_NPARAM, dtype=np.float64)
    o = _OFF["w1"][0]
    w1 = np.zeros((128, 80))
    w1[:, :67] = r.uniform(-1, 1, (128, 67)) * math.sqrt(6.0 / 67)
    p[o:o + w1.size] = w1.ravel()
    o = _OFF["w2"][0]
    p[o:o + 128 * 128] = (r.uniform(-1, 1, (128, 128)) * math.sqrt(6.0 / 128)).ravel()
    o = _OFF["w3"][0]
    p[o:o + 128] = r.uniform(-1, 1, 128) * math.sqrt(3.0 / 128)
    return p.astype(np.float16)


def run_workload(name, seed, scale, workdir, device=0, collect=0, params=None, threshold=0.0, full_threshold=0.0,
                 ext_budget=1, domain=None):
    """One whole job of a workload: (records, stats, pairs info, feature rows).  domain:
    the parameters the network was trained under (default: this workload's own)."""
    db, skip = workloads.generate(name, workdir, scale=scale, seed=seed)
    with Overlapper(workloads.params(name), device) as ov:
        ov.set_reads_seqdb(db)
        if skip:
            ov.set_skip_kmers(workloads.read_skip(skip))
        if params is not None:
            ov.set_filter(params, threshold, full_threshold, ext_budget,
                          domain=domain if domain is not None else training_domain(name))
        if collect:
            ov.collect_pairs(collect)
        ov.run()
        recs = ov.overlaps()
        st = ov.stats()
        info, feat = ov.pairs() if collect else (None, None)
    return recs, st, info, feat


def training_domain(name):
    """The filter domain of a workload: the overlapInCore parameters its network sees."""
    from . import filter_domain
    return filter_domain(workloads.WORKLOADS[name]["params"])


def read_errors(name):
    """The read error regime a workload's reads are generated with."""
    sy = workloads.WORKLOADS[name]["synth"]
    return f"{100 * sy['err']:g}% errors, sub:ins:del {sy['ratio']}"


def sample_weights(info, pos_weight=4.0):
    """Positives pos_weight; negatives 0.05 + their DP cells relative to the median
    negative that reached the DP (capped at 20)."""
    y = (info["overlaps"] > 0).astype(np.float32)
    cells = info["cells"].astype(np.float64)
    neg = (y == 0) & (cells > 0)
    med = float(np.median(cells[neg])) if neg.any() else 1.0
    w = np.where(y > 0, pos_weight, 0.05 + np.minimum(cells / max(med, 1.0), 20.0))
    return y, w.astype(np.float32)


class Trainer:
    """FP16 network with FP32 master weights on one GPU; all math in the library."""

    def __init__(self, params16, device=0):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        p = np.asarray(params16, dtype=np.float16)
        self.prm = torch.from_numpy(p.view(np.int16).copy()).to(self.dev)
        self.master = torch.from_numpy(p.astype(np.float32)).to(self.dev)
        self.m = torch.zeros_like(self.master)
        self.v = torch.zeros_like(self.master)
        self.grad = torch.zeros_like(self.master)
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self.step = 0

    def params(self):
        return self.prm.cpu().numpy().view(np.float16).copy()

    def _stream(self):
        return self.torch.cuda.current_stream(self.dev).cuda_stream

    def predict(self, X, batch=1 << 20):
        """Logits of every row of X (torch FP16 [n, 80] on the device)."""
        t = self.torch
        n = X.shape[0]
        out = t.empty(n, dtype=t.float32, device=self.dev)
        for i in range(0, n, batch):
            xb = X[i:i + batch].contiguous()
            mlp_forward(self.prm.data_ptr(), xb.data_ptr(), xb.shape[0], out[i:].data_ptr(), stream=self._stream())
        return out

    def fit(self, X, y, w, epochs=6, batch=32768, lr=2e-3, lr_min=2e-5, weight_decay=1e-5, seed=0, log=None):
        """Adam with a cosine learning-rate decay over all steps; returns mean losses per epoch."""
        t = self.torch
        n = X.shape[0]
        H1 = t.empty((batch, 128), dtype=t.float16, device=self.dev)
        H2 = t.empty_like(H1)
        G1 = t.empty_like(H1)
        G2 = t.empty_like(H1)
        logit = t.empty(batch, dtype=t.float32, device=self.dev)
        gen = t.Generator(device=self.dev)
        gen.manual_seed(seed)
        steps = epochs * ((n + batch - 1) // batch)
        k = 0
        hist = []
        st = self._stream()
        for ep in range(epochs):
            perm = t.randperm(n, generator=gen, device=self.dev)
            self.loss.zero_()
            wsum = 0.0
            for i in range(0, n, batch):
                idx = perm[i:i + batch]
                b = idx.shape[0]
                xb = X.index_select(0, idx).contiguous()
                yb = y.index_select(0, idx).contiguous()
                wb = w.index_select(0, idx).contiguous()
                lr_t = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * k / max(steps, 1)))
                mlp_forward(self.prm.data_ptr(), xb.data_ptr(), b, logit.data_ptr(), H1.data_ptr(), H2.data_ptr(),
                            stream=st)
                mlp_backward(self.prm.data_ptr(), xb.data_ptr(), H1.data_ptr(), H2.data_ptr(), logit.data_ptr(),
                             yb.data_ptr(), wb.data_ptr(), b, self.grad.data_ptr(), G1.data_ptr(), G2.data_ptr(),
                             self.loss.data_ptr(), stream=st)
                self.step += 1
                mlp_adam(self.master.data_ptr(), self.m.data_ptr(), self.v.data_ptr(), self.grad.data_ptr(),
                         self.prm.data_ptr(), lr_t, 0.9, 0.999, 1e-8, 1.0 / b, weight_decay, self.step, stream=st)
                k += 1
            wsum = float(w.sum().item())
            hist.append(float(self.loss.item()) / max(wsum, 1e-9))
            if log:
                log(f"epoch {ep + 1}/{epochs}: weighted loss {hist[-1]:.5f}")
        t.cuda.synchronize(self.dev)
        return hist


def choose_threshold(logit, label, recall):
    """Probability threshold that keeps at least `recall` of the positives."""
    pos = np.sort(np.asarray(logit, dtype=np.float64)[np.asarray(label) > 0])
    if len(pos) == 0:
        return 0.0
    k = int(math.floor((1.0 - recall) * len(pos)))
    cut = pos[min(k, len(pos) - 1)] - 1e-3   # keep every positive scored at or above pos[k]
    return float(1.0 / (1.0 + math.exp(-cut)))


def _logit(p):
    return -np.inf if p <= 0 else math.log(p / (1 - p))


def policy_cost(info, logit, t_drop, t_full, budget=1):
    """(recall, DP cells, pairs kept) of the two-threshold policy replayed on collected
    pairs: dropped pairs cost nothing and lose their overlaps; pairs below t_full stop
    once `budget` extensions found nothing, so they lose the overlaps found later
    (firstHit >= budget) and cost their first extension plus, for budget > 1, the mean
    cost of their later extensions times the extra ones run."""
    y = info["overlaps"] > 0
    fh = info["firstHit"]
    cells = info["cells"].astype(np.float64)
    first = info["cellsFirst"].astype(np.float64)
    ext = info["extensions"].astype(np.float64)
    z = np.asarray(logit, dtype=np.float32)
    keep = ~(z < np.float32(_logit(t_drop)))
    single = keep & (z < np.float32(_logit(t_full)))
    later = (cells - first) / np.maximum(ext - 1, 1)
    capped = first + np.maximum(np.minimum(ext, budget) - 1, 0) * later
    found_early = y & (fh >= 0) & (fh < budget)
    cost = np.where(single & ~found_early, capped, cells)[keep].sum()
    lost = (y & ~keep).sum() + (single & y & (fh >= budget)).sum()
    return 1.0 - lost / max(y.sum(), 1), float(cost), int(keep.sum())


def choose_thresholds(info, logit, recall_drop, recall_total, budget=1):
    """t_drop keeps recall_drop of the positives; t_full is the lowest cut (the most
    pairs on the extension budget) whose replayed recall still reaches recall_total."""
    y = info["overlaps"] > 0
    t_drop = choose_threshold(logit, y, recall_drop)
    z = np.asarray(logit, dtype=np.float64)
    kept = z[z >= _logit(t_drop)]
    best = None
    for q in np.concatenate([[0.0], np.linspace(0.5, 0.999, 60), [1.0]]):
        zc = np.quantile(kept, q) if q < 1.0 else np.inf
        t_full = 0.0 if q == 0.0 else (1.0 if not np.isfinite(zc) else float(1 / (1 + math.exp(-zc))))
        if t_full >= 1.0:
            t_full = 0.999999
        rec, cost, _ = policy_cost(info, logit, t_drop, t_full if q > 0 else t_drop, budget)
        if rec >= recall_total and (best is None or cost < best[1]):
            best = (t_full if q > 0 else t_drop, cost, rec)
    if best is None:   # the budget tier costs too much recall: full extension for every kept pair
        return t_drop, t_drop
    return t_drop, best[0]


def record_keys(rec):
    """(a_iid, b_iid, flipped) of each record -- the overlap checker's key.  flipped is
    bit 58 of the first data word (ovOverlap.H), i.e. bit 26 of record word 2."""
    rec = np.asarray(rec, dtype=np.uint32).reshape(-1, 6)
    flipped = (rec[:, 2] >> 26) & 1
    return (rec[:, 0].astype(np.uint64) << np.uint64(33)) | (rec[:, 1].astype(np.uint64) << np.uint64(1)) | \
        flipped.astype(np.uint64)


def compare(plain, filt):
    """Recall of the filtered records against the plain ones, and whether every
    filtered record equals its plain record word for word."""
    a = sort_records(plain)
    b = sort_records(filt)
    sa = set(bytes(r) for r in a)
    exact = all(bytes(r) in sa for r in b)
    ka, kb = np.unique(record_keys(a)), np.unique(record_keys(b))
    recall = len(np.intersect1d(ka, kb)) / max(len(ka), 1)
    return recall, exact


def evaluate(params, threshold, name="c2", seed=6, scale=1.0, workdir="/tmp/oic_filter", device=0,
             full_threshold=None, budget=1, pairs=True, domain=None):
    """Plain vs filtered run of one read set; returns a dict of the measured figures.
    pairs=False skips the pair-level figures (a third run collecting every pair).
    domain: the parameters the network was trained under (default: the workload's)."""
    if full_threshold is None:
        full_threshold = threshold
    out = {}
    if pairs:
        _, _, info, _ = run_workload(name, seed, scale, workdir, device, collect=1, params=params, threshold=0.0,
                                     domain=domain)
        y = info["overlaps"] > 0
        rec_replay, _, kept = policy_cost(info, info["score"], threshold, full_threshold, budget)
        keep = ~(info["score"] < np.float32(_logit(threshold)))
        cells_neg = info["cells"][~y].astype(np.float64)
        out = {"pairs": int(len(info)), "positives": int(y.sum()), "kept": int(keep.sum()),
               "pair_recall_drop_only": float((keep & y).sum() / max(y.sum(), 1)),
               "precision": float((keep & y).sum() / max(keep.sum(), 1)),
               "recall_replayed": float(rec_replay),
               "dropped_negative_cells_frac": float(cells_neg[~keep[~y]].sum() / max(cells_neg.sum(), 1))}
        del info
    rp, sp, _, _ = run_workload(name, seed, scale, workdir, device)
    rf, sf, _, _ = run_workload(name, seed, scale, workdir, device, params=params, threshold=threshold,
                                full_threshold=full_threshold, ext_budget=budget, domain=domain)
    recall, exact = compare(rp, rf)
    mk = lambda recs, s: {
        "overlaps": int(len(recs)), "ms": s["msTotal"], "ms_align": s["msAlign"], "dp_cells": int(s["dpCells"]),
        "overlaps_per_s": len(recs) / (s["msTotal"] / 1e3), "dp_cells_per_s": s["dpCells"] / (s["msTotal"] / 1e3)}
    f = mk(rf, sf)
    f.update({"ms_filter": sf["msFilter"], "filtered_pairs": int(sf["filteredPairs"])})
    return {
        **out,
        "thresholds": {"drop": threshold, "full": full_threshold, "budget": budget},
        "plain": mk(rp, sp), "filter": f,
        "recall": recall, "records_exact": bool(exact),
        "dp_cells_skipped_frac": 1.0 - sf["dpCells"] / max(sp["dpCells"], 1),
        "speedup": sp["msTotal"] / max(sf["msTotal"], 1e-9),
    }


def save(path, params, threshold, full_threshold, meta, budget=1):
    np.savez(path, params=np.asarray(params, dtype=np.float16), threshold=np.float64(threshold),
             full_threshold=np.float64(full_threshold), budget=np.int64(budget), meta=np.array(json.dumps(meta)))


def load(path):
    """(params float16[FILTER_NPARAM], drop threshold, full threshold, meta dict); the
    extension budget is meta["budget"], the parameters the network was trained under
    meta["domain"] (kmerLen, minOlapLen, maxErate) and the training reads' error regime
    meta["read_errors"]."""
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    if "domain" not in meta:
        raise ValueError(f"{path}: the filter file does not name the parameters it was trained under")
    meta["budget"] = int(z["budget"]) if "budget" in z else 1
    return z["params"].astype(np.float16), float(z["threshold"]), float(z["full_threshold"]), meta


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--train-seeds", default="1,2,3,4,5")
    ap.add_argument("--eval-seed", type=int, default=6)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--batch", type=int, default=32768)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--recall-drop", type=float, default=0.99998)
    ap.add_argument("--recall", type=float, default=0.9995)
    ap.add_argument("--budget", type=int, default=2, help="extensions without an overlap in the budget tier")
    ap.add_argument("--pos-weight", type=float, default=4.0)
    ap.add_argument("--init-seed", type=int, default=0)
    ap.add_argument("--workdir", default="/tmp/oic_filter")
    ap.add_argument("--out", default=None)
    ap.add_argument("--report", default=None)
    ap.add_argument("--also-eval", default="", help="more read sets to evaluate on, e.g. c5:5 (workload:seed)")
    a = ap.parse_args(argv)
    import torch

    def log(msg):
        print(f"[{time.strftime('%H:%M:%S')}] {msg}", flush=True)

    dev = torch.device("cuda", 0)
    Xs, ys, ws, info_all = [], [], [], []
    t0 = time.time()
    for s in [int(x) for x in a.train_seeds.split(",") if x]:
        recs, st, info, feat = run_workload(a.workload, s, a.scale, a.workdir, collect=1)
        y, w = sample_weights(info, a.pos_weight)
        log(f"seed {s}: {len(recs)} overlaps, {len(info)} pairs ({int(y.sum())} positive), "
            f"{st['dpCells']} DP cells, {st['msTotal']:.0f} ms")
        Xs.append(torch.from_numpy(feat.view(np.int16)).to(dev))
        ys.append(torch.from_numpy(y).to(dev))
        ws.append(torch.from_numpy(w).to(dev))
        info_all.append(info)
    X = torch.cat(Xs).view(torch.float16)
    y = torch.cat(ys)
    w = torch.cat(ws)
    del Xs, ys, ws
    log(f"labels collected in {time.time() - t0:.0f} s: {X.shape[0]} pairs")

    tr = Trainer(init_params(a.init_seed))
    t1 = time.time()
    torch.cuda.synchronize()
    hist = tr.fit(X, y, w, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.init_seed, log=log)
    train_s = time.time() - t1
    n = X.shape[0]
    flops = 3 * 2 * (80 * 128 + 128 * 128 + 128) * n * a.epochs
    log(f"trained {a.epochs} epochs in {train_s:.1f} s ({n * a.epochs / train_s / 1e6:.1f} M samples/s, "
        f"{flops / train_s / 1e12:.2f} TFLOP/s)")
    logit = tr.predict(X).cpu().numpy()
    yl = y.cpu().numpy()
    info = np.concatenate(info_all)
    thr, full = choose_thresholds(info, logit, a.recall_drop, a.recall, a.budget)
    rec_tr, cost_tr, kept_tr = policy_cost(info, logit, thr, full, a.budget)
    params = tr.params()
    meta = {"workload": a.workload, "scale": a.scale, "train_seeds": a.train_seeds, "epochs": a.epochs,
            "batch": a.batch, "lr": a.lr, "recall_drop_train": a.recall_drop, "recall_target_train": a.recall,
            "pos_weight": a.pos_weight, "train_pairs": int(n), "train_positives": int(yl.sum()), "loss": hist,
            "train_seconds": train_s, "train_samples_per_s": n * a.epochs / train_s,
            "train_tflops": flops / train_s / 1e12, "train_recall_replayed": rec_tr,
            "train_cells_left_frac": cost_tr / float(info["cells"].astype(np.float64).sum()),
            "train_pairs_kept": kept_tr, "budget": a.budget, "domain": training_domain(a.workload),
            "read_errors": read_errors(a.workload)}
    log(f"thresholds: drop {thr:.6g}, full {full:.6g}; training replay: recall {rec_tr:.5f}, "
        f"cells left {meta['train_cells_left_frac']:.4f}, pairs kept {kept_tr}")
    if a.out:
        save(a.out, params, thr, full, meta, a.budget)
        log(f"wrote {a.out}")
    del X, y, w
    torch.cuda.empty_cache()
    ev = evaluate(params, thr, a.workload, a.eval_seed, a.scale, a.workdir, full_threshold=full, budget=a.budget)
    log(json.dumps(ev))
    more = {}
    for spec in [s for s in a.also_eval.split(",") if s]:
        wl, sd = spec.split(":")
        more[spec] = evaluate(params, thr, wl, int(sd), 1.0, a.workdir, full_threshold=full, budget=a.budget,
                              pairs=False)
        log(spec + " " + json.dumps(more[spec]))
    if a.report:
        with open(a.report, "w") as f:
            json.dump({"meta": meta, "threshold": thr, "full_threshold": full, "budget": a.budget,
                       "eval_seed": a.eval_seed, "eval": ev, "also": more}, f, indent=1)


if __name__ == "__main__":
    main()
