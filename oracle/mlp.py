"""CPU oracle of the learned proposal's network (test infrastructure only).

Restates in numpy what the library's tensor-core kernels compute, with the
same BF16 rounding points, so their outputs and gradients can be checked:

* forward: x, h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2) enter the matrix
  products as BF16 (round to nearest even), weights as BF16, products
  accumulated in wide precision, biases added in FP32;
* proposal: q_b = (1 - 1/64) softmax(z_0..31)_b + 1/64 / 32 as the CDF knots
  C_1..C_31, and P = sigmoid(z_32);
* loss per record (bin b, plain trial count k):
  -log softmax(z)_b - (k - 1) log(1 - P) - log P, averaged;
* backward: dz, the masked dh2 and dh1 enter the products as BF16; bias
  gradients are the column sums of those BF16 values.

`grad_exact` is the same gradient in float64 without any rounding (checked
against finite differences), so the BF16 mirror's formulas are themselves
pinned.  The parameter vector layout is W1[64][8], b1[64], W2[64][64], b2[64],
W3[33][64], b3[33] (6881 floats).  The proposal is the one this project
defines; the sampler it feeds is get_positions_loop's rejection loop
(cmc_evolution_thr.c:855-926).
"""
import numpy as np

NIN, NH, NOUT, NBINS = 8, 64, 33, 32
FLOOR = 1.0 / 64.0
P_W1 = 0
P_B1 = P_W1 + NH * NIN
P_W2 = P_B1 + NH
P_B2 = P_W2 + NH * NH
P_W3 = P_B2 + NH
P_B3 = P_W3 + NOUT * NH
NPARAM = P_B3 + NOUT


def bf16(x):
    """Round float32 values to BF16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    a = (a + 0x7FFF + ((a >> 16) & 1)) >> 16 << 16
    return a.astype(np.uint32).view(np.float32).reshape(np.shape(x))


def unpack(w):
    w = np.asarray(w)
    return (w[P_W1:P_B1].reshape(NH, NIN), w[P_B1:P_W2], w[P_W2:P_B2].reshape(NH, NH), w[P_B2:P_W3],
            w[P_W3:P_B3].reshape(NOUT, NH), w[P_B3:NPARAM])


def pack(W1, b1, W2, b2, W3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3]).astype(np.float32)


def _mm(a, b):
    """Product of BF16-valued float32 arrays, accumulated in float64, rounded to float32."""
    return (a.astype(np.float64) @ b.astype(np.float64)).astype(np.float32)


def forward(w, feat):
    """Logits (n x 33) and the activations the backward pass needs."""
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(w, dtype=np.float32))
    x = bf16(feat)
    pre1 = _mm(x, bf16(W1).T) + b1
    h1 = bf16(np.maximum(pre1, 0.0))
    pre2 = _mm(h1, bf16(W2).T) + b2
    h2 = bf16(np.maximum(pre2, 0.0))
    z = _mm(h2, bf16(W3).T) + b3
    return z, (x, pre1, h1, pre2, h2)


def proposal(z):
    """CDF knots C_1..C_31 and P (n x 32), as the inference kernel stores them."""
    z = np.asarray(z, dtype=np.float64)
    e = np.exp(z[:, :NBINS] - z[:, :NBINS].max(axis=1, keepdims=True))
    q = (1.0 - FLOOR) * e / e.sum(axis=1, keepdims=True) + FLOOR / NBINS
    out = np.empty((z.shape[0], NBINS))
    out[:, :NBINS - 1] = np.cumsum(q[:, :NBINS - 1], axis=1)
    out[:, NBINS - 1] = 1.0 / (1.0 + np.exp(-z[:, NBINS]))
    return out


def _softplus(x):
    return np.maximum(x, 0.0) + np.log1p(np.exp(-np.abs(x)))


def loss_terms(z, bins, ntrial):
    """Per-record bin loss and trial-count loss (float64)."""
    z = np.asarray(z, dtype=np.float64)
    zb = z[:, :NBINS]
    mx = zb.max(axis=1, keepdims=True)
    lse = mx[:, 0] + np.log(np.exp(zb - mx).sum(axis=1))
    nll = lse - zb[np.arange(len(z)), bins]
    k = np.asarray(ntrial, dtype=np.float64)
    geo = (k - 1.0) * _softplus(z[:, NBINS]) + _softplus(-z[:, NBINS])
    return nll, geo


def _dz(z, bins, ntrial):
    z = np.asarray(z, dtype=np.float64)
    n = len(z)
    zb = z[:, :NBINS]
    s = np.exp(zb - zb.max(axis=1, keepdims=True))
    s /= s.sum(axis=1, keepdims=True)
    dz = np.zeros((n, NOUT))
    dz[:, :NBINS] = s
    dz[np.arange(n), bins] -= 1.0
    P = 1.0 / (1.0 + np.exp(-z[:, NBINS]))
    dz[:, NBINS] = np.asarray(ntrial, dtype=np.float64) * P - 1.0
    return dz / n


def grad_bf16(w, feat, bins, ntrial):
    """Mean gradient with the kernels' BF16 rounding points, and the mean losses."""
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(w, dtype=np.float32))
    z, (x, pre1, h1, pre2, h2) = forward(w, feat)
    dz = bf16(_dz(z, bins, ntrial).astype(np.float32))
    gW3 = _mm(dz.T, h2)
    gb3 = dz.astype(np.float64).sum(axis=0)
    dh2 = _mm(dz, bf16(W3))
    dh2 = bf16(np.where(pre2 > 0, dh2, 0.0).astype(np.float32))
    gW2 = _mm(dh2.T, h1)
    gb2 = dh2.astype(np.float64).sum(axis=0)
    dh1 = _mm(dh2, bf16(W2))
    dh1 = bf16(np.where(pre1 > 0, dh1, 0.0).astype(np.float32))
    gW1 = _mm(dh1.T, x)
    gb1 = dh1.astype(np.float64).sum(axis=0)
    nll, geo = loss_terms(z, bins, ntrial)
    return pack(gW1, gb1, gW2, gb2, gW3, gb3), (nll.mean(), geo.mean())


def _forward_exact(w, feat):
    W1, b1, W2, b2, W3, b3 = (np.asarray(a, np.float64) for a in unpack(w))
    x = np.asarray(feat, np.float64)
    pre1 = x @ W1.T + b1
    h1 = np.maximum(pre1, 0.0)
    pre2 = h1 @ W2.T + b2
    h2 = np.maximum(pre2, 0.0)
    return h2 @ W3.T + b3, (x, pre1, h1, pre2, h2)


def loss_exact(w, feat, bins, ntrial):
    z, _ = _forward_exact(w, feat)
    nll, geo = loss_terms(z, bins, ntrial)
    return float(nll.mean() + geo.mean())


def grad_exact(w, feat, bins, ntrial):
    """Mean gradient in float64 without rounding (back-propagation)."""
    W1, b1, W2, b2, W3, b3 = (np.asarray(a, np.float64) for a in unpack(w))
    z, (x, pre1, h1, pre2, h2) = _forward_exact(w, feat)
    dz = _dz(z, bins, ntrial)
    dh2 = (dz @ W3) * (pre2 > 0)
    dh1 = (dh2 @ W2) * (pre1 > 0)
    return np.concatenate([(dh1.T @ x).ravel(), dh1.sum(0), (dh2.T @ h1).ravel(), dh2.sum(0),
                           (dz.T @ h2).ravel(), dz.sum(0)])


def adam_step(w, m, v, g, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (float32), as the library applies it."""
    w, m, v, g = (np.asarray(a, np.float32).copy() for a in (w, m, v, g))
    m = np.float32(b1) * m + np.float32(1 - b1) * g
    v = np.float32(b2) * v + np.float32(1 - b2) * g * g
    c1 = np.float32(1 - b1 ** t)
    c2 = np.float32(1 - b2 ** t)
    w = w - np.float32(lr) * (m / c1) / (np.sqrt(v / c2) + np.float32(eps))
    return w, m, v


def init_params(seed=1):
    """A random parameter vector (uniform +-sqrt(6 / fan_in); small output layer)."""
    rng = np.random.default_rng(seed)
    W1 = rng.uniform(-1, 1, (NH, NIN)) * np.sqrt(6.0 / NIN)
    W2 = rng.uniform(-1, 1, (NH, NH)) * np.sqrt(6.0 / NH)
    W3 = rng.uniform(-1, 1, (NOUT, NH)) * 0.3 * np.sqrt(6.0 / NH)
    b1 = rng.uniform(-0.1, 0.1, NH)
    b2 = rng.uniform(-0.1, 0.1, NH)
    b3 = rng.uniform(-0.1, 0.1, NOUT)
    return pack(W1, b1, W2, b2, W3, b3)


def sample_index(seed, step, pos, n):
    """Record drawn for batch position pos of training step `step` (the
    library's SplitMix64-style hash; vectorised over pos)."""
    M = (1 << 64) - 1
    pos = np.asarray(pos, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (np.uint64(seed & M) + np.uint64(0x9E3779B97F4A7C15) *
             ((np.uint64(step) << np.uint64(32)) + pos + np.uint64(1)))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z % np.uint64(n)).astype(np.int64)
