"""The learned densification proposal on the GPU (no reference counterpart: the
reference densifies by its gradient threshold alone, src/shaders/densify.wgsl,
which stays the fallback).

The model's tensor-core kernels against a NumPy restatement of the same BF16
arithmetic (inference, on tcgen05, within 1e-3; the training kernel's weight and bias
gradient values tensor by tensor; one AdamW step moves every weight with a
clear gradient by lr against that gradient's sign), training on a separable rule, and
the trainer: a model that is never confident reproduces the plain rule exactly,
one that vetoes everything stops every clone and split, and the log labels
every clone/split candidate."""

from __future__ import annotations

import math

import numpy as np
import pytest

from diorama_gb300 import DEFAULT_SETTINGS, DensifyMLP, RawGaussians, Trainer
from diorama_gb300.training import MLP_FEATURES, MLP_PARAMS
from dataclasses import replace

from test_gpu_training import ring_views, scrambled_start, truth_scene

pytestmark = pytest.mark.gpu

erf = np.vectorize(math.erf)


def bf16(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(w):
    o = 0
    shapes = [("W1", (12, 64)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (64, 2)), ("b3", (2,))]
    out = {}
    for name, shape in shapes:
        size = int(np.prod(shape))
        out[name] = w[o:o + size].reshape(shape).astype(np.float64)
        o += size
    out["mean"] = w[o:o + 12].astype(np.float64)
    out["inv_std"] = w[o + 12:o + 24].astype(np.float64)
    return out


def gelu(x):
    return 0.5 * x * (1 + erf(x / math.sqrt(2)))


def gelu_grad(x):
    return 0.5 * (1 + erf(x / math.sqrt(2))) + x * np.exp(-0.5 * x * x) / math.sqrt(2 * math.pi)


def forward(p, features):
    x = bf16(((features - p["mean"]) * p["inv_std"]).astype(np.float32)).astype(np.float64)
    z1 = x @ bf16(p["W1"]).astype(np.float64) + p["b1"]
    a1 = bf16(gelu(z1)).astype(np.float64)
    z2 = a1 @ bf16(p["W2"]).astype(np.float64) + p["b2"]
    a2 = bf16(gelu(z2)).astype(np.float64)
    z3 = a2 @ bf16(p["W3"]).astype(np.float64) + p["b3"]
    return x, z1, a1, z2, a2, z3


def random_weights(rng, scale=0.3):
    w = rng.normal(0, scale, MLP_PARAMS + 24).astype(np.float32)
    w[MLP_PARAMS:MLP_PARAMS + 12] = rng.normal(0, 0.5, 12)
    w[MLP_PARAMS + 12:] = rng.uniform(0.5, 2.0, 12)
    return w


@pytest.mark.parametrize("count", [1, 127, 128, 129, 1000, 100_003])
def test_predict_matches_bf16_restatement(device, count):
    """Inference runs on tcgen05 (128 candidates a CTA, accumulators in tensor
    memory): full, partial and single-candidate tiles, and many CTAs at once."""
    rng = np.random.default_rng(3)
    mlp = DensifyMLP(device, seed=1)
    w = random_weights(rng)
    mlp.setWeights(w)
    assert np.array_equal(mlp.weights(), w)
    features = rng.normal(0, 1.5, (count, MLP_FEATURES)).astype(np.float32)
    got = mlp.predictHost(features)
    z3 = forward(unpack(w), features)[-1]
    want = 1 / (1 + np.exp(z3[:, 0] - z3[:, 1]))
    assert got.shape == (count,) and np.abs(got - want).max() <= 1e-3
    assert device.check() == 0  # no product's wait gave up
    mlp.destroy()


def restated_gradient(p, features, labels):
    """The mean cross-entropy's gradient in float64, rounding to BF16 where the
    kernel does: the normalized inputs, the weights, the activations, and the
    deltas that enter tensor-core products (dZ3 into dA2, dZ2 into dA1, and all
    three in the weight gradients); bias gradients sum the unrounded deltas."""
    b = lambda v: bf16(np.asarray(v, np.float32)).astype(np.float64)  # noqa: E731
    x, z1, a1, z2, a2, z3 = forward(p, features)
    prob = np.exp(z3 - z3.max(1, keepdims=True))
    prob /= prob.sum(1, keepdims=True)
    d3 = (prob - np.eye(2)[labels]) / len(labels)
    d2 = (b(d3) @ b(p["W3"]).T) * gelu_grad(z2)
    d1 = (b(d2) @ b(p["W2"]).T) * gelu_grad(z1)
    return np.concatenate([(x.T @ b(d1)).ravel(), d1.sum(0), (a1.T @ b(d2)).ravel(), d2.sum(0),
                           (a2.T @ b(d3)).ravel(), d3.sum(0)])


def test_weight_gradients_match_float64_restatement(device):
    """The training kernel's gradient values (not only their signs) against the
    float64 restatement, tensor by tensor: the largest error within 1% of the
    tensor's largest gradient, and the element-wise relative error over the
    gradients above 5% of it small (BF16 operands, FP32 accumulation)."""
    rng = np.random.default_rng(4)
    mlp = DensifyMLP(device, seed=2)
    w = random_weights(rng, 0.2)
    mlp.setWeights(w)
    features = rng.normal(0, 1.0, (1000, MLP_FEATURES)).astype(np.float32)
    labels = (rng.random(1000) < 0.4).astype(np.uint8)
    got = mlp.gradient(features, labels).astype(np.float64)
    assert np.array_equal(mlp.weights(), w)  # nothing updated
    want = restated_gradient(unpack(w), features, labels)
    sizes = [("W1", 12 * 64), ("b1", 64), ("W2", 64 * 64), ("b2", 64), ("W3", 128), ("b3", 2)]
    o = 0
    report = {}
    for name, size in sizes:
        g, r = got[o:o + size], want[o:o + size]
        o += size
        scale = np.abs(r).max()
        big = np.abs(r) > 0.05 * scale
        rel = np.abs(g[big] - r[big]) / np.abs(r[big])
        report[name] = (float(np.abs(g - r).max() / scale), float(np.median(rel)), float(rel.max()))
        assert report[name][0] <= 1e-2 and report[name][1] <= 2e-3 and report[name][2] <= 5e-2, report
    # The same gradient once more: the kernel clears its accumulators.
    assert np.allclose(mlp.gradient(features, labels), got, rtol=1e-5, atol=1e-7 * np.abs(got).max())
    mlp.destroy()


def test_one_adamw_step_follows_the_gradient(device):
    """Adam's first step moves each weight by lr against its gradient's sign
    (m / (1 - beta1) = g, v / (1 - beta2) = g^2)."""
    rng = np.random.default_rng(4)
    mlp = DensifyMLP(device, seed=2)
    w = random_weights(rng, 0.2)
    mlp.setWeights(w)
    features = rng.normal(0, 1.0, (256, MLP_FEATURES)).astype(np.float32)
    labels = (rng.random(256) < 0.5).astype(np.uint8)
    mlp.train(features, labels, epochs=1, batch=256, lr=1e-4, weightDecay=0.0)
    after = mlp.weights()
    p = unpack(w)
    # Training sets the normalization from the samples first.
    mean = features.astype(np.float64).mean(0)
    var = ((features.astype(np.float64) - mean) ** 2).mean(0)
    p["mean"] = mean.astype(np.float32).astype(np.float64)
    p["inv_std"] = (1 / np.sqrt(var + 1e-12)).astype(np.float32).astype(np.float64)
    grads = restated_gradient(p, features, labels)
    step = after[:MLP_PARAMS].astype(np.float64) - w[:MLP_PARAMS]
    clear = np.abs(grads) > 0.05 * np.abs(grads).max()
    agree = np.mean(np.sign(step[clear]) == -np.sign(grads[clear]))
    assert clear.sum() > 200 and agree >= 0.98, (clear.sum(), agree)
    assert np.allclose(np.abs(step[clear]), 1e-4, rtol=1e-2), np.abs(step[clear]).max()
    mlp.destroy()


def test_training_learns_a_separable_rule(device):
    rng = np.random.default_rng(5)
    f = rng.normal(0, 1, (24000, MLP_FEATURES)).astype(np.float32)
    y = (f[:, 0] + 0.5 * f[:, 3] - 0.7 * f[:, 8] > 0.2).astype(np.uint8)
    mlp = DensifyMLP(device, seed=3)
    losses = mlp.train(f[:20000], y[:20000], epochs=8, batch=512, lr=3e-3, weightDecay=0.01, seed=1)
    assert losses[-1] < losses[0] and losses[-1] < 0.2, losses
    acc = np.mean((mlp.predictHost(f[20000:]) >= 0.5) == (y[20000:] == 1))
    assert acc >= 0.95, acc
    mlp.destroy()


def _densifying_run(device, views, params, log=False):
    settings = replace(DEFAULT_SETTINGS, extent=3.85, densifyFrom=100, densifyUntil=1000, densifyInterval=100,
                       densifyGradThreshold=5e-5, opacityResetInterval=100000)
    t = Trainer(device, RawGaussians(params, np.zeros(params.size // 16 * 45, np.float32)), views, settings)
    if log:
        t.setDensifyLog(True, 300)
    for _ in range(1000):
        t.step()
    return t


def test_densify_log_labels_every_candidate(device):
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)
    t = _densifying_run(device, views, params, log=True)
    tallies = [(d.cloned, d.split) for d in t.densifications]
    assert sum(c + s for c, s in tallies) > 0, tallies
    # Every clone/split candidate logged, labelled once 300 steps have passed.
    f, y, pending = t.takeDensifySamples()
    logged = sum(c + s for d, (c, s) in zip(t.densifications, tallies) if d.step + 300 <= 1000)
    assert len(y) == logged and set(np.unique(y)) <= {0, 1} and np.isfinite(f).all()
    assert pending == sum(c + s for c, s in tallies) - logged
    assert 0 < y.mean() < 1
    t.destroy()


def test_learned_densify_fallback_and_veto(device):
    """One densification of the same state three ways: plain, with a model that is
    never confident (every output exactly 0.5: the plain rule, bit for bit), and
    with one that always predicts the children's death (no clone, no split)."""
    truth, random = truth_scene()
    views = ring_views(device, truth)
    params = scrambled_start(truth, random)
    warm = _densifying_run(device, views, params)
    raw = warm.exportRaw()
    stats = warm.buffers["stats"].read(np.float32)
    moments = warm.readMoments()
    n = raw.params.size // 16
    rng = np.random.default_rng(9)
    stats = stats.reshape(-1, 4)
    stats[:, 1] = np.maximum(stats[:, 1], 1)
    stats[:, 0] = stats[:, 1] * rng.uniform(0, 2e-4, n)  # about half the Gaussians above the threshold
    stats = stats.reshape(-1)
    warm.destroy()

    def densify_once(mlp=None):
        t = Trainer(device, RawGaussians(raw.params.copy(), raw.sh.copy()), views,
                    replace(DEFAULT_SETTINGS, extent=3.85, densifyGradThreshold=1e-4))
        t.writeMoments(moments)
        t.buffers["stats"].write(stats)
        if mlp is not None:
            t.setDensifyMLP(mlp, 0.6)
        t.iteration = 700
        t.densify(False)
        d = t.densifications[0]
        out = (d.removed, d.kept, d.cloned, d.split), t.exportRaw().params, t.densifyMLPStats
        t.destroy()
        return out

    plain, plain_params, _ = densify_once()
    assert plain[2] + plain[3] > 50, plain
    unsure = DensifyMLP(device)
    unsure.setWeights(np.concatenate([np.zeros(MLP_PARAMS, np.float32), np.zeros(12, np.float32),
                                      np.ones(12, np.float32)]))
    same, same_params, stats_unsure = densify_once(unsure)
    assert same == plain and np.array_equal(same_params, plain_params)
    assert stats_unsure == {"scored": plain[2] + plain[3], "confident": 0, "vetoed": 0}
    w = np.zeros(MLP_PARAMS + 24, np.float32)
    w[MLP_PARAMS - 2:MLP_PARAMS] = [10.0, -10.0]  # b3: P(survive) = sigmoid(-20)
    w[MLP_PARAMS + 12:] = 1.0
    veto = DensifyMLP(device)
    veto.setWeights(w)
    none, _, stats_veto = densify_once(veto)
    assert none[2] == 0 and none[3] == 0 and none[0] == plain[0]
    assert stats_veto["vetoed"] == stats_veto["scored"] == plain[2] + plain[3]
    unsure.destroy()
    veto.destroy()
