"""GPU tests of the MLP radiance cache kernels (BF16 tensor-core forward,
backward and Adam) against the CPU FP64 reference of the oracle.

The GPU computes with BF16 weights/activations and FP32 accumulation, so the
reference is evaluated in FP64 on the same BF16-rounded weights and the same
(BF16) encoded inputs; the remaining difference is the BF16 rounding of hidden
activations and gradients.  Tolerance: 1e-2 relative (norm-wise), as specified
for the learned part."""
import numpy as np
import pytest

import oracle as O
import snkpt
from snkpt import scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-2


def bf16(x):
    """Round float32 values to BF16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    a = (a + 0x7FFF + ((a >> 16) & 1)) & 0xFFFF0000
    return a.astype(np.uint32).view(np.float32).astype(np.float64)


def records(rng, n, lo, hi):
    r = np.zeros((n, 16), np.float32)
    r[:, 0:3] = rng.uniform(lo, hi, (n, 3))
    r[:, 3] = rng.uniform(0.1, 1.0, n)
    d = rng.normal(size=(n, 3)); d /= np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.normal(size=(n, 3)); nn /= np.linalg.norm(nn, axis=1, keepdims=True)
    r[:, 4:7] = d
    r[:, 7] = (rng.uniform(size=n) < 0.2).astype(np.float32)
    r[:, 8:11] = nn
    r[:, 12:15] = rng.uniform(0.2, 0.8, (n, 3))
    return r


def encode_ref(r, lo, hi):
    """float64 restatement of the 64-feature encoding."""
    n = r.shape[0]
    f = np.zeros((n, 64))
    p = np.clip((r[:, 0:3].astype(np.float64) - lo) / (hi - lo), 0, 1)
    for a in range(3):
        for k in range(6):
            f[:, 12 * a + 2 * k] = np.sin(2.0 ** k * np.pi * p[:, a])
            f[:, 12 * a + 2 * k + 1] = np.cos(2.0 ** k * np.pi * p[:, a])
    d, nn = r[:, 4:7].astype(np.float64), r[:, 8:11].astype(np.float64)
    for a in range(3):
        f[:, 36 + 2 * a] = np.sin(np.pi * d[:, a]); f[:, 37 + 2 * a] = np.cos(np.pi * d[:, a])
        f[:, 42 + 2 * a] = np.sin(np.pi * nn[:, a]); f[:, 43 + 2 * a] = np.cos(np.pi * nn[:, a])
    f[:, 48:51] = d; f[:, 51:54] = nn
    f[:, 54] = r[:, 3]; f[:, 55:58] = r[:, 12:15]; f[:, 58] = r[:, 7]
    f[:, 59] = np.sum(d * nn, 1)
    m = r[:, 7:8].astype(np.float64)
    f[:, 60:63] = 0.04 * (1 - m) + r[:, 12:15] * m
    f[:, 63] = 1.0
    return f


@pytest.fixture(scope="module")
def tracer(cuda, built_lib):
    pt = snkpt.PathTracer(0)
    lo, hi = np.array([-10.0, 0.0, -20.0]), np.array([30.0, 15.0, 20.0])
    pt.cache_set_bounds(lo, hi)
    return pt, lo, hi


def nrel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def test_encoding_matches_reference(tracer):
    pt, lo, hi = tracer
    r = records(np.random.default_rng(1), 4096, lo, hi)
    f = pt.cache_encode(r)
    ref = encode_ref(r, lo, hi)
    assert np.abs(f - ref).max() < 1e-2      # BF16 rounding (8 bits of mantissa)
    assert np.array_equal(f, bf16(f))        # the values are exactly BF16


def test_forward_matches_fp64(tracer):
    pt, lo, hi = tracer
    pt.cache_reset(3)
    w = pt.cache_get_weights()
    r = records(np.random.default_rng(2), 8192, lo, hi)
    y = pt.cache_infer(r)
    ref = O.mlp_forward(bf16(w), pt.cache_encode(r).astype(np.float64))
    assert nrel(y, ref) < RTOL


def test_gradient_matches_fp64(tracer):
    pt, lo, hi = tracer
    pt.cache_reset(4)
    w = pt.cache_get_weights()
    rng = np.random.default_rng(3)
    r = records(rng, 4096, lo, hi)
    s = np.zeros((4096, 20), np.float32)
    s[:, :16] = r
    s[:, 16:19] = rng.uniform(0.0, 2.0, (4096, 3))
    s[:, 19] = (rng.uniform(size=4096) < 0.9).astype(np.float32)
    loss, g = pt.cache_train(s, lr=0.0, want_grad=True)
    x = pt.cache_encode(r).astype(np.float64)
    ref_loss, ref_g = O.mlp_grad(bf16(w), x, s[:, 16:19], s[:, 19])
    assert abs(loss - ref_loss) <= RTOL * abs(ref_loss)
    assert nrel(g, ref_g) < RTOL
    for l in range(5):   # per layer as well
        a, b = (l * 4096, (l + 1) * 4096) if l < 4 else (4 * 4096, 4 * 4096 + 192)
        assert nrel(g[a:b], ref_g[a:b]) < RTOL, l
    # lr = 0 leaves the weights unchanged
    assert np.array_equal(pt.cache_get_weights(), w)


def test_adam_step_matches_reference(tracer):
    pt, lo, hi = tracer
    pt.cache_reset(5)
    w0 = pt.cache_get_weights().astype(np.float64)
    rng = np.random.default_rng(4)
    s = np.zeros((2048, 20), np.float32)
    s[:, :16] = records(rng, 2048, lo, hi)
    s[:, 16:19] = rng.uniform(0.0, 2.0, (2048, 3))
    s[:, 19] = 1.0
    _, g = pt.cache_train(s, lr=1e-2, want_grad=True)
    w1 = pt.cache_get_weights()
    W, m, v = w0.copy(), np.zeros_like(w0), np.zeros_like(w0)
    O.mlp_adam(W, m, v, g.astype(np.float64), 1, lr=1e-2)
    assert np.abs(w1 - W).max() < 1e-5


def test_training_is_deterministic_and_learns(tracer):
    pt, lo, hi = tracer
    rng = np.random.default_rng(6)
    batches = []
    for _ in range(40):
        r = records(rng, 4096, lo, hi)
        s = np.zeros((4096, 20), np.float32)
        s[:, :16] = r
        # smooth synthetic radiance: depends on position, normal and albedo
        p = (r[:, 0:3] - lo) / (hi - lo)
        base = 0.5 + 0.4 * np.sin(3 * p[:, 0:1]) * np.cos(2 * p[:, 2:3]) + 0.3 * r[:, 9:10]
        s[:, 16:19] = np.clip(base * r[:, 12:15] * 2.0, 0.0, None)
        s[:, 19] = 1.0
        batches.append(s)
    losses = []
    for run in range(2):
        pt.cache_reset(7)
        ls = [pt.cache_train(b, lr=1e-2)[0] for b in batches]
        losses.append(ls)
        if run == 0:
            w_first = pt.cache_get_weights()
    assert losses[0] == losses[1]
    assert np.array_equal(w_first, pt.cache_get_weights())
    assert np.mean(losses[0][-5:]) < 0.1 * np.mean(losses[0][:3])
