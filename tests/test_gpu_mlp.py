"""tcgen05 BF16 GEMM kernels of the surrogate against torch (GPU).

Reference: the same BF16 operands multiplied in FP32 by torch.  Tolerances:
FP32 outputs 1e-5 relative to the row's magnitude (accumulation order), BF16
outputs 1e-2 (one BF16 rounding).
"""
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu


def rel(a, b):
    import torch
    return float(((a.float() - b.float()).abs().max() / b.float().abs().max().clamp_min(1e-30)))


@pytest.mark.parametrize("M,N,K", [(300, 256, 64), (128, 64, 256), (1000, 256, 256), (77, 32, 16)])
def test_linear_forward_matches_torch(cuda_device, M, N, K):
    import torch
    ops = pkg("mlp_ops")
    torch.manual_seed(0)
    X = torch.randn(M, K, device=cuda_device).bfloat16()
    W = (torch.randn(N, K, device=cuda_device) / K ** 0.5).bfloat16()
    b = torch.randn(N, device=cuda_device)
    Y32 = torch.empty(M, N, device=cuda_device)
    ops.linear(X, W, bias=b, Y32=Y32)
    ref = X.float() @ W.float().t() + b
    assert ops.status() == 0
    assert rel(Y32, ref) < 1e-5
    Y = torch.empty(M, N, device=cuda_device, dtype=torch.bfloat16)
    YT = torch.zeros(N, M, device=cuda_device, dtype=torch.bfloat16)
    Z = torch.empty(M, N, device=cuda_device, dtype=torch.bfloat16)
    cs = torch.zeros(N, device=cuda_device)
    ops.linear(X, W, bias=b, act=True, Y=Y, YT=YT, Z=Z, colsum=cs)
    act = torch.nn.functional.silu(ref)
    assert rel(Y, act) < 1e-2
    assert rel(YT.t(), act) < 1e-2
    assert rel(Z, ref) < 1e-2
    assert rel(cs, act.sum(0)) < 1e-4


def test_linear_dgrad_silu_derivative(cuda_device):
    import torch
    ops = pkg("mlp_ops")
    torch.manual_seed(1)
    M, N, K = 256, 256, 256
    dZ = torch.randn(M, K, device=cuda_device).bfloat16()
    Wt = (torch.randn(N, K, device=cuda_device) / 16).bfloat16()
    zp = torch.randn(M, N, device=cuda_device).bfloat16()
    out = torch.empty(M, N, device=cuda_device, dtype=torch.bfloat16)
    cs = torch.zeros(N, device=cuda_device)
    ops.linear(dZ, Wt, zprev=zp, Y=out, colsum=cs)
    z = zp.float()
    s = torch.sigmoid(z)
    ref = (dZ.float() @ Wt.float().t()) * (s * (1 + z * (1 - s)))
    assert rel(out, ref) < 1e-2
    assert rel(cs, ref.sum(0)) < 1e-4


@pytest.mark.parametrize("Mo,No,Kb", [(256, 64, 4096), (64, 256, 1024), (256, 256, 65536)])
def test_wgrad_matches_torch(cuda_device, Mo, No, Kb):
    import torch
    ops = pkg("mlp_ops")
    torch.manual_seed(2)
    A = torch.randn(Mo, Kb, device=cuda_device).bfloat16()
    B = torch.randn(No, Kb, device=cuda_device).bfloat16()
    C = torch.zeros(Mo, No, device=cuda_device)
    ops.wgrad(A, B, C)
    ref = A.float() @ B.float().t()
    assert ops.status() == 0
    assert rel(C, ref) < 1e-5


@pytest.mark.parametrize("M", [1, 127, 128, 4097, 300000])
def test_fused_forward_matches_layer_by_layer(cuda_device, M):
    """pjg_mlp_forward (all five layers in one launch, activations on chip,
    weights streamed by bulk copies) equals the layer-by-layer tcgen05 forward:
    the same BF16 roundings at the same points."""
    import torch
    sg = pkg("surrogate")
    net = sg.MLP(cuda_device, seed=7)
    g = torch.Generator(device=cuda_device).manual_seed(3)
    for b in net.b:
        b.copy_(0.1 * torch.randn(b.shape, generator=g, device=cuda_device))
    net.refresh()
    X = torch.randn(M, 64, generator=g, device=cuda_device).to(torch.bfloat16)
    X[:, 54:] = 0
    ref = net.forward(X.contiguous())
    got = net.infer(X.contiguous())
    torch.cuda.synchronize()
    assert pkg("mlp_ops").status() == 0
    err = ((got - ref).abs() / (ref.abs() + 1e-2)).max().item()
    assert err < 1e-3, err
