"""Learned-CDF MLP: the hand-written GPU forward/backward against a float64
CPU reference (itself checked by finite differences)."""
import ctypes as C

import numpy as np
import pytest

KIN, KH = 48, 64


def unpack(p):
    o = 0
    W1 = p[o:o + KIN * KH].reshape(KH, KIN); o += KIN * KH
    b1 = p[o:o + KH]; o += KH
    W2 = p[o:o + KH * KH].reshape(KH, KH); o += KH * KH
    b2 = p[o:o + KH]; o += KH
    w3 = p[o:o + KH]; o += KH
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def loss_and_grad(p, X, t):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    y = h2 @ w3 + b3
    e = y - t
    n = len(t)
    loss = float(np.mean(e * e))
    dy = 2 * e / n
    g_w3 = h2.T @ dy
    g_b3 = dy.sum()
    d2 = np.outer(dy, w3) * (a2 > 0)
    g_W2 = d2.T @ h1
    g_b2 = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    g_W1 = d1.T @ X
    g_b1 = d1.sum(0)
    g = np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_w3, [g_b3]])
    return loss, g


def sample(seed, n):
    rng = np.random.default_rng(seed)
    npar = KIN * KH + KH + KH * KH + KH + KH + 1
    p = rng.normal(0, 0.2, size=npar)
    X = rng.integers(0, 2, size=(n, KIN)).astype(np.float64)
    t = rng.random(n)
    return p, X, t


def test_reference_gradient_finite_difference():
    p, X, t = sample(1, 64)
    _, g = loss_and_grad(p, X, t)
    rng = np.random.default_rng(2)
    for i in rng.choice(len(p), size=40, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (loss_and_grad(pp, X, t)[0] - loss_and_grad(pm, X, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i])


@pytest.mark.gpu
@pytest.mark.parametrize("n", [100, 1000, 4096])
def test_gpu_gradients_match_float64(gpu, n):
    L = gpu.lib()
    L.kite_mlp_grad_check.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_uint32, C.POINTER(C.c_float),
                                                                  C.POINTER(C.c_float)]
    npar = L.kite_mlp_param_count()
    assert L.kite_mlp_input_count() == KIN
    p, X, t = sample(n, n)
    assert npar == len(p)
    p32, X32, t32 = p.astype(np.float32), X.astype(np.float32), t.astype(np.float32)
    g_out = np.zeros(npar, dtype=np.float32)
    l_out = np.zeros(1, dtype=np.float32)
    f = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    assert L.kite_mlp_grad_check(f(p32), f(np.ascontiguousarray(X32)), f(t32), n, f(g_out), f(l_out)) == 0
    loss, g = loss_and_grad(p32.astype(np.float64), X32.astype(np.float64), t32.astype(np.float64))
    # float32 accumulation in a different order: relative 1e-3 of the gradient scale
    scale = np.abs(g).max()
    assert np.abs(g_out - g).max() <= 1e-3 * scale + 1e-7
    assert abs(l_out[0] - loss) <= 1e-4 * max(1.0, loss)


@pytest.mark.gpu
def test_learned_splitters_beat_histogram_on_skewed_keys(gpu):
    """The gain of the trained network over the method without it: on keys
    whose top bits are heavily skewed (an AT-rich low-complexity genome,
    k=63), the sampled-histogram splitters cannot cut inside a heavy bin and
    leave the key ranges badly unbalanced; the learned CDF spreads each bin's
    mass and cuts inside it.  Counts are identical either way."""
    from kite_gb300 import synth
    fq = synth.skewed_workload(seed=4, n_reads=25_000)
    res = {}
    for name, mode in (("sampled", gpu.SPLIT_SAMPLED), ("learned", gpu.SPLIT_LEARNED)):
        with gpu.Counter(63, True, 2, splitter_mode=mode, imbalance_bound=100.0) as c:
            c.submit(fq)
            out = c.finish()
            res[name] = (out, c.stats())
    (out_s, st_s), (out_l, st_l) = res["sampled"], res["learned"]
    assert st_l["splitter_used"] == gpu.SPLIT_LEARNED and st_s["splitter_used"] == gpu.SPLIT_SAMPLED
    assert [(m["partition_id"], p) for m, p in out_s] == [(m["partition_id"], p) for m, p in out_l]
    assert st_s["tiles_per_bucket"] >= 512
    # measured range imbalance: sampled ~18, learned ~3.5
    assert st_s["range_imbalance"] > 8.0
    assert st_l["range_imbalance"] < 0.4 * st_s["range_imbalance"]
