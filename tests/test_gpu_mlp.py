"""Learned CDF (an autoregressive masked MLP over the key bits): the
hand-written GPU forward/backward against a float64 CPU reference (itself
checked by finite differences), and the gain of the trained network over
the histogram splitters."""
import ctypes as C

import numpy as np
import pytest

KIN, KH, KB0 = 48, 64, 16
KOUT = KIN - KB0
NPAR = KIN * KH + KH + KH * KH + KH + KOUT * KH + KOUT


def masks():
    """Autoregressive masks: hidden unit k has degree 16 + k//2; first-layer
    unit j sees inputs i < deg(j), second-layer unit k sees first-layer units
    of degree <= deg(k), output o (bit 16 + o) sees second-layer units of
    degree <= 16 + o."""
    deg = KB0 + np.arange(KH) // 2
    m1 = (np.arange(KIN)[None, :] < deg[:, None]).astype(np.float64)
    m2 = (deg[None, :] <= deg[:, None]).astype(np.float64)
    m3 = (deg[None, :] <= (KB0 + np.arange(KOUT))[:, None]).astype(np.float64)
    return m1, m2, m3


def unpack(p):
    o = 0
    W1 = p[o:o + KIN * KH].reshape(KH, KIN); o += KIN * KH
    b1 = p[o:o + KH]; o += KH
    W2 = p[o:o + KH * KH].reshape(KH, KH); o += KH * KH
    b2 = p[o:o + KH]; o += KH
    W3 = p[o:o + KOUT * KH].reshape(KOUT, KH); o += KOUT * KH
    b3 = p[o:o + KOUT]
    return W1, b1, W2, b2, W3, b3


def bits(views):
    return ((views[:, None] >> np.arange(KIN - 1, -1, -1, dtype=np.uint64)[None, :]) & np.uint64(1)).astype(np.float64)


def loss_and_grad(p, views):
    """Mean binary cross-entropy of bits 16..47 given the bits above, and its
    gradient (float64; masked weights get zero gradient)."""
    m1, m2, m3 = masks()
    W1, b1, W2, b2, W3, b3 = unpack(p)
    W1, W2, W3 = W1 * m1, W2 * m2, W3 * m3
    X = bits(views)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    z = h2 @ W3.T + b3
    y = X[:, KB0:]
    n = len(views)
    loss = float(np.mean(np.maximum(z, 0) - y * z + np.log1p(np.exp(-np.abs(z)))))
    dz = (1 / (1 + np.exp(-z)) - y) / (n * KOUT)
    g_W3 = (dz.T @ h2) * m3
    g_b3 = dz.sum(0)
    d2 = (dz @ W3) * (a2 > 0)
    g_W2 = (d2.T @ h1) * m2
    g_b2 = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    g_W1 = (d1.T @ X) * m1
    g_b1 = d1.sum(0)
    g = np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_W3.ravel(), g_b3])
    return loss, g


def sample(seed, n):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.2, size=NPAR)
    m1, m2, m3 = masks()
    live = np.concatenate([m1.ravel(), np.ones(KH), m2.ravel(), np.ones(KH), m3.ravel(), np.ones(KOUT)])
    p = p * live  # masked weights are zero, as the library keeps them
    views = rng.integers(0, 1 << 48, size=n, dtype=np.uint64)
    return p, views


def test_reference_gradient_finite_difference():
    p, views = sample(1, 64)
    _, g = loss_and_grad(p, views)
    rng = np.random.default_rng(2)
    for i in rng.choice(len(p), size=60, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (loss_and_grad(pp, views)[0] - loss_and_grad(pm, views)[0]) / (2 * h)
        m1, m2, m3 = masks()
        live = np.concatenate([m1.ravel(), np.ones(KH), m2.ravel(), np.ones(KH), m3.ravel(), np.ones(KOUT)])
        if live[i]:
            assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i])
        else:
            assert g[i] == 0.0 and abs(fd) <= 1e-9  # a masked weight changes nothing


def test_outputs_see_only_higher_bits():
    # the autoregressive property: flipping bit i changes no output for bits <= i
    p, views = sample(3, 16)
    m1, m2, m3 = masks()
    W1, b1, W2, b2, W3, b3 = unpack(p)

    def logits(v):
        X = bits(v)
        h1 = np.maximum(X @ (W1 * m1).T + b1, 0)
        h2 = np.maximum(h1 @ (W2 * m2).T + b2, 0)
        return h2 @ (W3 * m3).T + b3
    base = logits(views)
    for i in range(KIN):
        flipped = logits(views ^ np.uint64(1 << (KIN - 1 - i)))
        for o in range(KOUT):
            if KB0 + o <= i:
                assert np.array_equal(flipped[:, o], base[:, o])


@pytest.mark.gpu
@pytest.mark.parametrize("n", [100, 1000, 4096])
def test_gpu_gradients_match_float64(gpu, n):
    L = gpu.lib()
    L.kite_mlp_grad_check.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_uint64), C.c_uint32,
                                      C.POINTER(C.c_float), C.POINTER(C.c_float)]
    assert L.kite_mlp_param_count() == NPAR
    assert L.kite_mlp_input_count() == KIN
    p, views = sample(n, n)
    p32 = p.astype(np.float32)
    g_out = np.zeros(NPAR, dtype=np.float32)
    l_out = np.zeros(1, dtype=np.float32)
    f = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    assert L.kite_mlp_grad_check(f(p32), views.ctypes.data_as(C.POINTER(C.c_uint64)), n, f(g_out), f(l_out)) == 0
    loss, g = loss_and_grad(p32.astype(np.float64), views)
    # float32 accumulation in a different order: relative 1e-3 of the gradient scale
    scale = np.abs(g).max()
    assert np.abs(g_out - g).max() <= 1e-3 * scale + 1e-7
    assert abs(l_out[0] - loss) <= 1e-4 * max(1.0, loss)
    assert np.all(g_out[g == 0] == 0)  # masked weights get no gradient


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
    assert st_s["range_imbalance"] > 8.0
    assert st_l["range_imbalance"] < 0.2 * st_s["range_imbalance"]
    assert st_l["mlp_pred_imbalance"] < 1.5
