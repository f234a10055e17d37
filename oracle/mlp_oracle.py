"""CPU oracle of the learned start vector model (test infrastructure only):
numpy restatement of the forward pass, the loss and the backward pass that
the GPU library runs in propack_gb300/csrc/pgb_mlp.cu, with the same
parameter layout (W1[256][18], b1, W2[256][256] as [out][in], b2, w3, b3)
and, when ``bf16=True``, the same BF16 rounding points (weights, the two
hidden activations and the layer-2 output gradient), so that the GPU
gradients can be checked entry by entry.  With ``bf16=False`` everything is
FP64, which is what the finite-difference check of the formulas uses.
"""
import numpy as np

IN, H = 18, 256
OW1 = 0
OB1 = OW1 + H * IN
OW2 = OB1 + H
OB2 = OW2 + H * H
OW3 = OB2 + H
OB3 = OW3 + H
NP = OB3 + 1
EPS = 1e-4


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float32."""
    x = np.asarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OW1:OB1].reshape(H, IN), p[OB1:OW2], p[OW2:OB2].reshape(H, H), p[OB2:OW3], p[OW3:OB3], p[OB3])


def forward(p, F, bf=True):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    r = (lambda x: bf16(x).astype(np.float64)) if bf else (lambda x: np.asarray(x, dtype=np.float64))
    W1b, W2b, w3b = r(W1), r(W2), r(w3)
    F = np.asarray(F, dtype=np.float64)
    H1 = r(np.maximum(F @ W1b.T + b1, 0.0))
    H2 = r(np.maximum(H1 @ W2b.T + b2, 0.0))
    out = H2 @ w3b + b3
    return out, (F, W1b, W2b, w3b, H1, H2)


def loss_and_grad(p, F, U, bf=True):
    """(loss, flat gradient) of L(u0) = -(1/k) sum_j log(c_j^2 + eps N / k)
    + log N, N = ||u0||^2, c = U' u0, u0 = the network's output."""
    out, (F, W1b, W2b, w3b, H1, H2) = forward(p, F, bf)
    if bf:
        out = out.astype(np.float32).astype(np.float64)
    U = np.asarray(U, dtype=np.float64)
    k = U.shape[1]
    c = U.T @ out
    N = out @ out
    eps = EPS * N / k
    d = c * c + eps
    loss = np.log(N) - np.sum(np.log(d)) / k
    coef = -2.0 * c / (d * k)
    ck = 2.0 / N - 2.0 * np.sum((EPS / k) / d) / k
    g = U @ coef + ck * out
    if bf:
        g = g.astype(np.float32).astype(np.float64)
    r = (lambda x: bf16(x).astype(np.float64)) if bf else (lambda x: x)
    dw3 = H2.T @ g
    db3 = g.sum()
    D2 = r(g[:, None] * w3b[None, :] * (H2 > 0))
    dW2 = D2.T @ H1
    db2 = D2.sum(0)
    D1 = (D2 @ W2b) * (H1 > 0)
    dW1 = D1.T @ F
    db1 = D1.sum(0)
    grad = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]])
    return loss, grad


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(NP)
    p[OW1:OB1] = rng.standard_normal(H * IN) * np.sqrt(2.0 / IN)
    p[OW2:OB2] = rng.standard_normal(H * H) * np.sqrt(2.0 / H)
    p[OW3:OB3] = rng.standard_normal(H) * np.sqrt(1.0 / H)
    return p
