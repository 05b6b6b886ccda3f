"""The surrogate's weight packing for the fused tcgen05 forward, on the CPU:
every W[n][k] lands at the byte the C ABI documents for pjg_mlp_forward,
((n / 8) * (K / 8) + k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2."""
import numpy as np
import pytest

from conftest import pkg

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("N,K", [(256, 64), (256, 256), (64, 256), (8, 8), (24, 40)])
def test_pack_core_layout(N, K):
    W = torch.randn(N, K).to(torch.bfloat16)
    packed = pkg("mlp_ops").pack_core(W).contiguous()
    raw = packed.view(torch.int16).numpy().reshape(-1)  # 2-byte elements
    bits = W.view(torch.int16).numpy()
    n, k = np.meshgrid(np.arange(N), np.arange(K), indexing="ij")
    byte = ((n // 8) * (K // 8) + k // 8) * 128 + (n % 8) * 16 + (k % 8) * 2
    assert packed.numel() == N * K
    assert np.array_equal(raw[byte // 2], bits)
