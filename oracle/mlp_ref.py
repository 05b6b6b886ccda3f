"""CPU reference of the surrogate network's forward and backward passes.

TEST INFRASTRUCTURE ONLY: checks the tcgen05 forward / input-gradient /
weight-gradient kernels (pyjac-v2_gb300/csrc/pjg_mlp.cu) as used by
surrogate.MLP.  Emulates the kernels' precision: BF16 inputs, weights and
stored activations (round-to-nearest-even), FP32 accumulation, so that the
only differences left are accumulation order and the rare BF16 rounding flip
they cause.
"""
import numpy as np


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even); returns float32."""
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(X, Ws, bs):
    """X [M, K0] (already BF16-valued); Ws [out, in]; returns outputs and saved (Z, A)."""
    a = bf16(X)
    saved = []
    for l in range(len(Ws) - 1):
        z = a @ bf16(Ws[l]).T.astype(np.float32) + bs[l]
        A = bf16(silu(z))
        saved.append((bf16(z), A, a))
        a = A
    y = a @ bf16(Ws[-1]).T.astype(np.float32) + bs[-1]
    saved.append((None, None, a))
    return y.astype(np.float32), saved


def backward(dY, Ws, saved):
    """Weight/bias gradients for the BF16-emulated network (FP32 math)."""
    L = len(Ws)
    gW = [None] * L
    gb = [None] * L
    dZ = bf16(dY)
    gb[L - 1] = dY.sum(0)
    for l in range(L - 1, -1, -1):
        a_in = saved[l][2]
        gW[l] = dZ.T.astype(np.float64) @ a_in.astype(np.float64)
        if l > 0:
            z = saved[l - 1][0].astype(np.float32)
            s = 1.0 / (1.0 + np.exp(-z))
            dA = dZ @ bf16(Ws[l]).astype(np.float32)
            dz = dA * (s * (1.0 + z * (1.0 - s)))
            gb[l - 1] = dz.sum(0)
            dZ = bf16(dz)
    return gW, gb
