"""torch-tensor wrappers of the tcgen05 MLP kernels (pjg_mlp_linear / pjg_mlp_wgrad).

All operands are contiguous CUDA tensors: BF16 activations/weights, FP32
biases, gradients and outputs.  Calls are asynchronous on the current torch
stream.  There is no fallback: a missing library or an unsupported shape
raises.
"""
import ctypes

import torch

from . import _lib


def _ptr(t):
    return None if t is None else t.data_ptr()


def _ld(t):
    return 0 if t is None else t.stride(0)


def _check(t, dtype, name):
    if t is None:
        return
    if not (t.is_cuda and t.dtype == dtype and t.dim() == 2 and t.stride(1) == 1):
        raise ValueError("%s must be a CUDA %s matrix with unit column stride" % (name, dtype))


def linear(X, W, bias=None, act=False, zprev=None, Y=None, YT=None, Z=None, Y32=None, colsum=None):
    """Y = act(X W^T + b) [* SiLU'(zprev)]; X [M, K] bf16, W [N, K] bf16.

    Fills the provided outputs (Y bf16 [M, N], YT bf16 [N, >=M], Z bf16 [M, N],
    Y32 fp32 [M, N], colsum fp32 [N] accumulated) and returns them.
    """
    lib = _lib.load()
    _check(X, torch.bfloat16, "X")
    _check(W, torch.bfloat16, "W")
    for t, n in ((Y, "Y"), (YT, "YT"), (Z, "Z"), (zprev, "zprev")):
        _check(t, torch.bfloat16, n)
    _check(Y32, torch.float32, "Y32")
    M, K = X.shape
    N = W.shape[0]
    if W.shape[1] != K:
        raise ValueError("W must be [N, K]")
    st = torch.cuda.current_stream(X.device).cuda_stream
    _lib.check("pjg_mlp_linear", lib.pjg_mlp_linear(
        _ptr(X), _ld(X), _ptr(W), _ld(W), M, N, K, _ptr(bias), int(bool(act)), _ptr(zprev),
        _ld(zprev), _ptr(Y), _ld(Y), _ptr(YT), _ld(YT), _ptr(Z), _ld(Z), _ptr(Y32), _ld(Y32),
        _ptr(colsum), st))
    return Y, YT, Z, Y32


def wgrad(A, B, C):
    """C += A B^T with A [Mo, Kb] bf16, B [No, Kb] bf16, C [Mo, No] fp32."""
    lib = _lib.load()
    _check(A, torch.bfloat16, "A")
    _check(B, torch.bfloat16, "B")
    _check(C, torch.float32, "C")
    Mo, Kb = A.shape
    No = B.shape[0]
    st = torch.cuda.current_stream(A.device).cuda_stream
    _lib.check("pjg_mlp_wgrad", lib.pjg_mlp_wgrad(
        _ptr(A), _ld(A), _ptr(B), _ld(B), Mo, No, Kb, _ptr(C), _ld(C), st))
    return C


def pack_core(W):
    """BF16 [N, K] -> the core-matrix layout of pjg_mlp_forward (N, K multiples of 8):
    8-row x 16-byte blocks, row-group major, then K."""
    N, K = W.shape
    return W.to(torch.bfloat16).reshape(N // 8, 8, K // 8, 8).permute(0, 2, 1, 3).contiguous()


def forward_fused(X, Wp, b, Y=None):
    """The whole network in one tcgen05 launch: X [M, 64] bf16, Wp the five
    packed weights (pack_core), b the five FP32 biases -> Y [M, 64] fp32."""
    lib = _lib.load()
    _check(X, torch.bfloat16, "X")
    M = X.shape[0]
    if Y is None:
        Y = torch.empty(M, 64, dtype=torch.float32, device=X.device)
    W = (ctypes.c_void_p * 5)(*[w.data_ptr() for w in Wp])
    B = (ctypes.c_void_p * 5)(*[x.data_ptr() for x in b])
    st = torch.cuda.current_stream(X.device).cuda_stream
    _lib.check("pjg_mlp_forward", lib.pjg_mlp_forward(X.data_ptr(), X.stride(0), M, W, B,
                                                      Y.data_ptr(), Y.stride(0), st))
    return Y


def status(clear=True):
    """1 if a tensor-core kernel timed out waiting on its accumulator."""
    return int(_lib.load().pjg_mlp_status(int(bool(clear))))
