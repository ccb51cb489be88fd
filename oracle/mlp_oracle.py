"""CPU ORACLE of the surrogate MLP (test infrastructure only).

numpy restatement of the forward pass, the Poisson + multinomial loss and the
backward pass of photonpropagation.jl_gb300/csrc/pp_mlp.cu, in FP32 with the
same BF16 rounding points as the training kernels (inputs, weights, stored
activations, head gradient, hidden gradients), so that device gradients can be
checked tensor by tensor; the fused inference kernel rounds its forward pass
at the same points.  The surrogate has no counterpart in the reference, so this
oracle is pinned by finite differences of its own loss (tests/test_mlp.py).
"""
from __future__ import annotations

import numpy as np


def bf16(x: np.ndarray) -> np.ndarray:
    """Round FP32 to BF16 (nearest even) and back to FP32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


class MLPOracle:
    """Layers given as lists of padded (W [rows x cols], b [rows]) FP32 arrays."""

    def __init__(self, weights, biases, n_in, n_bins, round_bf16=True):
        # round_bf16=False runs everything in FP64 (for finite differences)
        self.dtype = np.float32 if round_bf16 else np.float64
        self.W = [np.asarray(w, self.dtype) for w in weights]
        self.b = [np.asarray(b, self.dtype) for b in biases]
        self.n_in = n_in
        self.n_bins = n_bins
        self.r = bf16 if round_bf16 else (lambda a: a)

    def forward(self, x):
        r = self.r
        in_pad = self.W[0].shape[1]
        X = np.zeros((x.shape[0], in_pad), self.dtype)
        X[:, :self.n_in] = x
        self.X0 = r(X)
        W16 = [r(w) for w in self.W]
        self.W16 = W16
        a = self.X0
        self.Z, self.Y = [], []
        for l in range(len(self.W) - 1):
            z = a @ W16[l].T + self.b[l]
            self.Z.append(r(z))
            a = r(silu(z))
            self.Y.append(a)
        self.O = a @ W16[-1].T + self.b[-1]
        return self.O

    def predict(self, x):
        """Expected count exp(min(o0, 30)) and the softmax time PDF, the outputs
        of the fused inference kernel."""
        O = self.forward(x)
        lam = np.exp(np.minimum(O[:, 0], 30.0))
        logits = O[:, 1:1 + self.n_bins]
        e = np.exp(logits - logits.max(axis=1, keepdims=True))
        return lam, e / e.sum(axis=1, keepdims=True)

    def loss_grad(self, x, count, hist):
        r = self.r
        O = self.forward(x)
        B = x.shape[0]
        nb = self.n_bins
        o0 = np.minimum(O[:, 0], 30.0)
        lam = np.exp(o0)
        logits = O[:, 1:1 + nb]
        mx = logits.max(axis=1, keepdims=True)
        e = np.exp(logits - mx)
        S = e.sum(axis=1, keepdims=True)
        p = e / S
        H = hist.sum(axis=1, keepdims=True)
        loss = np.sum(lam - count * o0) / B - np.sum(hist * (logits - mx - np.log(S))) / B
        dO = np.zeros_like(O)
        dO[:, 0] = (lam - count) / B
        dO[:, 1:1 + nb] = (H * p - hist) / B
        dO16 = r(dO)
        gW = [None] * len(self.W)
        gb = [None] * len(self.W)
        L = len(self.W) - 1
        gb[L] = dO.sum(axis=0)
        gW[L] = dO16.T @ self.Y[L - 1]
        dz = r((dO16 @ self.W16[L]) * silu_grad(self.Z[L - 1]))
        for l in range(L - 1, -1, -1):
            xin = self.Y[l - 1] if l > 0 else self.X0
            gb[l] = dz.sum(axis=0)
            gW[l] = dz.T @ xin
            if l == 0:
                break
            dz = r((dz @ self.W16[l]) * silu_grad(self.Z[l - 1]))
        return float(loss), gW, gb
