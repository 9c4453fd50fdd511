"""CPU checks of the learned-filter oracle (oracle/filter_oracle.py) and host logic."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import filter_oracle as fo  # noqa: E402

import canu_gb300 as oic  # noqa: E402
from canu_gb300 import filter_train  # noqa: E402


def _problem(n=64, seed=1):
    r = np.random.default_rng(seed)
    p = fo.init_params(seed).astype(np.float64)
    p[fo.OFF["b1"][0]:fo.OFF["b1"][0] + 128] = r.normal(0, 0.1, 128)
    p[fo.OFF["b2"][0]:fo.OFF["b2"][0] + 128] = r.normal(0, 0.1, 128)
    x = r.normal(0, 1, (n, fo.IN))
    x[:, 67:] = 0
    y = (r.random(n) < 0.3).astype(np.float64)
    w = r.uniform(0.5, 2.0, n)
    return p, x, y, w


def test_backward_matches_central_differences():
    p, x, y, w = _problem()
    z, h1, h2 = fo.forward(p, x, round_act=False)
    g, _ = fo.backward(p, x, h1, h2, z, y, w, round_grad=False)
    idx = [0, 5, 66, 128 * 80 - 14, fo.OFF["b1"][0] + 7, fo.OFF["w2"][0] + 77, fo.OFF["w2"][0] + 16000,
           fo.OFF["b2"][0] + 3, fo.OFF["w3"][0] + 9, fo.OFF["b3"][0]]
    ng = fo.numeric_grad(p, x, y, w, idx)
    np.testing.assert_allclose(g[idx], ng, rtol=1e-5, atol=1e-7)


def test_padding_inputs_get_no_gradient():
    p, x, y, w = _problem()
    z, h1, h2 = fo.forward(p, x)
    g, _ = fo.backward(p, x, h1, h2, z, y, w)
    gw1 = g[:128 * 80].reshape(128, 80)
    assert np.all(gw1[:, 67:] == 0)


def test_parameter_layout_agrees_with_binding():
    assert fo.NPARAM == oic.FILTER_NPARAM
    for k, (o, s) in fo.OFF.items():
        assert oic.FILTER_OFFSETS[k] == (o, s)
    assert filter_train.init_params(0).shape == (oic.FILTER_NPARAM,)
    # the product's initialiser keeps the padding columns at zero too
    w1 = filter_train.init_params(0)[:128 * 80].reshape(128, 80)
    assert np.all(w1[:, 67:] == 0) and np.any(w1[:, :67] != 0)


def test_features_of_a_true_overlap_and_a_repeat():
    k = 22
    # 10 kb dovetail on diagonal +5000 between two 15 kb reads: one bin, density ~ 0.8
    runs = [(5000 + s, 100 + k - 1, s) for s in range(0, 10000, 125)]
    f = fo.features(15000, 15000, 80 * 100, runs, k).astype(np.float32)
    b = ((5000 + 15000) * 64) // 30000
    assert f[b] > 0.7 and np.count_nonzero(f[:64]) == 1
    # a 2 kb shared repeat on the same diagonal: the same bin, a quarter of the density
    runs = [(9000 + s, 60 + k - 1, 4000 + s) for s in range(0, 2000, 100)]
    g = fo.features(15000, 15000, 20 * 60, runs, k).astype(np.float32)
    assert g[b] < 0.25 * f[b] + 0.05
    assert f[66] > g[66]
    assert np.all(f[67:] == 0) and np.all(g[67:] == 0)


def test_threshold_choice_keeps_the_requested_recall():
    r = np.random.default_rng(3)
    logit = r.normal(0, 2, 100000)
    label = (r.random(100000) < 0.2).astype(np.float32)
    for rec in (0.999, 0.9995, 0.99):
        t = filter_train.choose_threshold(logit, label, rec)
        z = np.float32(np.log(t / (1 - t)))
        kept = ~(logit.astype(np.float32) < z)
        got = (kept & (label > 0)).sum() / (label > 0).sum()
        assert got >= rec


def test_record_keys_read_the_flipped_bit():
    rec = np.zeros((2, 6), dtype=np.uint32)
    rec[:, 0], rec[:, 1] = 5, 9
    rec[1, 2] = 1 << 26
    k = filter_train.record_keys(rec)
    assert k[0] != k[1] and (k[1] & 1) == 1 and (k[0] & 1) == 0
    recall, exact = filter_train.compare(rec, rec[:1])
    assert recall == 0.5 and exact


def _fake_pairs():
    info = np.zeros(8, dtype=oic.PAIR_DTYPE)
    # positives found by the first extension, one found by a later one, negatives
    info["overlaps"] = [1, 1, 1, 0, 0, 0, 0, 1]
    info["firstHit"] = [0, 0, 0, -1, -1, -1, -1, 2]
    info["cells"] = [100, 100, 100, 1000, 1000, 50, 0, 300]
    info["cellsFirst"] = [100, 100, 100, 70, 70, 50, 0, 60]
    info["extensions"] = [1, 1, 1, 10, 10, 1, 0, 3]
    logit = np.array([3.0, 2.0, 1.0, 2.5, -1.0, -2.0, -3.0, 4.0], dtype=np.float32)
    return info, logit


def test_policy_replay_counts_dropped_and_single_extension_pairs():
    info, logit = _fake_pairs()
    sig = lambda z: float(1 / (1 + np.exp(-z)))
    # no filtering at all
    rec, cost, kept = filter_train.policy_cost(info, logit, 0.0, 0.0)
    assert rec == 1.0 and cost == info["cells"].sum() and kept == 8
    # drop below 0 (pairs 4, 5, 6), full extension for every kept pair
    rec, cost, kept = filter_train.policy_cost(info, logit, sig(0.0), sig(0.0))
    assert kept == 5 and rec == 1.0 and cost == 100 * 3 + 1000 + 300
    # single extension below 5: the late positive (pair 7) is lost, negative 3 costs 70
    rec, cost, kept = filter_train.policy_cost(info, logit, sig(0.0), sig(5.0))
    assert rec == 0.75 and cost == 300 + 70 + 60
    # full extension from 3.5 up keeps pair 7
    rec, cost, _ = filter_train.policy_cost(info, logit, sig(0.0), sig(3.5))
    assert rec == 1.0 and cost == 300 + 70 + 300
    # a budget of 2: pair 7 (found by its third extension) is still lost; pair 3 pays
    # one more extension at its mean later cost (930 / 9); a budget of 3 keeps pair 7
    rec, cost, _ = filter_train.policy_cost(info, logit, sig(0.0), sig(5.0), budget=2)
    assert rec == 0.75 and abs(cost - (300 + 70 + 930 / 9 + 60 + 120)) < 1e-9
    rec, cost, _ = filter_train.policy_cost(info, logit, sig(0.0), sig(5.0), budget=3)
    assert rec == 1.0 and abs(cost - (300 + 70 + 2 * 930 / 9 + 300)) < 1e-9


def test_threshold_pair_meets_the_training_recall():
    r = np.random.default_rng(5)
    n = 20000
    info = np.zeros(n, dtype=oic.PAIR_DTYPE)
    y = r.random(n) < 0.2
    info["overlaps"] = y
    info["firstHit"] = np.where(y, np.where(r.random(n) < 0.01, 1, 0), -1)
    info["cells"] = np.where(y, 1000, r.integers(0, 20000, n))
    info["cellsFirst"] = np.minimum(info["cells"], 800)
    logit = (np.where(y, 2.0, -1.0) + r.normal(0, 1.0, n)).astype(np.float32)
    t_drop, t_full = filter_train.choose_thresholds(info, logit, 0.999, 0.995)
    rec, cost, _ = filter_train.policy_cost(info, logit, t_drop, t_full)
    assert rec >= 0.995
    rec0, cost0, _ = filter_train.policy_cost(info, logit, t_drop, t_drop)
    assert cost <= cost0
