"""The surrogate's tensor-core GEMM (wc_nn_gemm: tcgen05, BF16 operands, FP32 accumulation) on
one GPU, timed with CUDA events beside PyTorch's matmul of the same tensors.

    python -m watercube_gb300.gemm [--shapes MxNxK,...] [--iters 20] [--warmup 3]

Each shape is C = relu(A B^T + bias) with A row-major (m x k), B^T output-major (n x k) and a
BF16 C, the form of the surrogate's edge-MLP layers. Prints one JSON object per shape: the mean
time per launch, TFLOP/s, and the GB/s of A read and C written (the bytes that bound these
shapes at n = 128).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

from . import _abi as A

DEFAULT_SHAPES = "1048576x128x128,1048576x128x384,262144x128x256"


def time_shape(m: int, n: int, k: int, iters: int, warmup: int, compare_torch: bool = True) -> dict:
    import torch

    lib = A.lib()
    gen = torch.Generator(device="cpu").manual_seed(0)
    a = torch.randn(m, k, generator=gen).to(torch.bfloat16).cuda()
    wt = torch.randn(n, k, generator=gen).to(torch.bfloat16).cuda()
    bias = torch.randn(n, generator=gen).cuda()
    c = torch.zeros(m, n, dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    g = A.GemmDesc()
    g.m, g.n, g.k = m, n, k
    g.k_chunk = ((k + 63) // 64) * 64
    g.a, g.lda, g.b, g.ldb = a.data_ptr(), k, wt.data_ptr(), k
    g.bias, g.relu, g.c_bf16, g.ldc = bias.data_ptr(), 1, c.data_ptr(), n
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def launch():
        A.check(lib.wc_nn_gemm(C.byref(g), err.data_ptr(), stream), "wc_nn_gemm")

    for _ in range(warmup):
        launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(iters):
        launch()
    e1.record()
    torch.cuda.synchronize()
    if int(err.item()) != 0:
        raise A.WatercubeError(A.WC_ERR_CUDA, f"wc_nn_gemm reported device error {int(err.item())}")
    ms = e0.elapsed_time(e1) / iters
    out = {"shape": f"{m}x{n}x{k}", "ms": ms, "tflops": 2.0 * m * n * k / ms / 1e9,
           "gbs_a_c": (m * k + m * n) * 2 / ms / 1e6}
    ref = torch.relu(a.float() @ wt.float().t() + bias)
    out["max_rel_err"] = float((c.float() - ref).abs().max() / (ref.abs().max() + 1e-6))
    if compare_torch:
        for _ in range(warmup):
            torch.relu(a @ wt.t() + bias).to(torch.bfloat16)
        e0.record()
        for _ in range(iters):
            torch.relu(a @ wt.t() + bias).to(torch.bfloat16)
        e1.record()
        torch.cuda.synchronize()
        out["torch_ms"] = e0.elapsed_time(e1) / iters
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--shapes", default=DEFAULT_SHAPES, help="comma-separated MxNxK")
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--no-torch", action="store_true", help="skip the PyTorch comparison")
    args = ap.parse_args(argv)
    A.check(A.lib().wc_set_device(0), "wc_set_device")
    for s in args.shapes.split(","):
        m, n, k = (int(v) for v in s.lower().split("x"))
        print(json.dumps(time_shape(m, n, k, args.iters, args.warmup, not args.no_torch)), flush=True)


if __name__ == "__main__":
    main()
