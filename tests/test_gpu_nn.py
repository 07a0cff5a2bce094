"""Tensor-core GEMM of the surrogate (tcgen05, BF16 operands, FP32 accumulation) against a plain
PyTorch FP32 matmul of the same BF16 inputs, in every operand and epilogue form the network
uses. Tolerance: 1e-3 of the output scale for FP32 outputs (FP32 sums of exact BF16 products in
a different order), plus one BF16 rounding (2^-8 relative) for BF16 outputs."""
import ctypes as C

import numpy as np
import pytest

from watercube_gb300 import _abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.fail("no CUDA device for a GPU test")
    return t


def run(lib, torch, **kw):
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    g = _abi.GemmDesc()
    for k, v in kw.items():
        setattr(g, k, v.data_ptr() if hasattr(v, "data_ptr") else v)
    if not g.k_chunk:
        g.k_chunk = ((g.k + 63) // 64) * 64
    torch.cuda.synchronize()
    rc = lib.wc_nn_gemm(C.byref(g), err.data_ptr(), None)
    assert rc == _abi.WC_OK, lib.wc_last_error().decode()
    torch.cuda.synchronize()
    assert int(err.item()) == 0


def rnd(torch, *shape, seed=0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(*shape, generator=g).to(torch.bfloat16).cuda()


def close(out, ref, rel=1e-3):
    scale = ref.abs().max().item() + 1e-6
    err = (out.float() - ref).abs().max().item()
    assert err <= rel * scale, f"max err {err:.3e} vs scale {scale:.3e}"


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (300, 128, 128), (1000, 128, 256), (257, 16, 32), (77, 200, 136)])
def test_plain_weight_gemm(wclib, torch, m, n, k):
    a = rnd(torch, m, k, seed=1)
    wt = rnd(torch, n, k, seed=2)  # B^T, output-major weights
    bias = torch.randn(n, device="cuda")
    c = torch.zeros(m, n, device="cuda")
    run(wclib, torch, m=m, n=n, k=k, a=a, lda=k, b=wt, ldb=k, bias=bias, c_f32=c, ldc=n)
    close(c, a.float() @ wt.float().t() + bias)


def test_concat_gather_relu_bf16(wclib, torch):
    m, n = 500, 128
    x = rnd(torch, 700, 128, seed=3)
    y = rnd(torch, 700, 128, seed=4)  # the row gather applies to both sources
    rows = torch.randint(0, 700, (m,), device="cuda", dtype=torch.int32)
    wt = rnd(torch, n, 256, seed=5)
    p = rnd(torch, 900, n, seed=6)
    q = rnd(torch, 900, n, seed=7)
    i1 = torch.randint(0, 900, (m,), device="cuda", dtype=torch.int32)
    i2 = torch.randint(0, 900, (m,), device="cuda", dtype=torch.int32)
    c = torch.zeros(m, n, device="cuda", dtype=torch.bfloat16)
    # A = [x[rows] | y[rows]]: columns 0..127 from x, 128..255 from y
    run(wclib, torch, m=m, n=n, k=256, a=x, lda=128, a_rows=rows, a2=y, lda2=128, k_split=128, b=wt, ldb=256,
        add1=p, add1_idx=i1, add2=q, add2_idx=i2, ld_add=n, relu=1, c_bf16=c, ldc=n)
    a = torch.cat([x[rows.long()].float(), y[rows.long()].float()], dim=1)
    ref = torch.relu(a @ wt.float().t() + p[i1.long()].float() + q[i2.long()].float())
    close(c, ref, rel=8e-3)


def test_input_gradient_form(wclib, torch):
    # dX = dY . W^T with W stored [k_in x n_out] row-major, i.e. B = W^T given row-major
    m, k_in, n_out = 384, 256, 128
    dy = rnd(torch, m, n_out, seed=8)
    w = rnd(torch, k_in, n_out, seed=9)
    c = torch.zeros(m, k_in, device="cuda")
    run(wclib, torch, m=m, n=k_in, k=n_out, a=dy, lda=n_out, b=w, ldb=n_out, c_f32=c, ldc=k_in)
    close(c, dy.float() @ w.float().t())


def test_weight_gradient_split_k(wclib, torch):
    # dW = X^T dY over 5,000 rows: A transposed, B row-major, split in 4 K ranges
    rows, k_in, n_out = 5000, 128, 128
    x = rnd(torch, rows, k_in, seed=10)
    dy = rnd(torch, rows, n_out, seed=11)
    chunk = 1280
    splits = (rows + chunk - 1) // chunk
    part = torch.zeros(splits, k_in, n_out, device="cuda")
    run(wclib, torch, m=k_in, n=n_out, k=rows, k_chunk=chunk, a=x, lda=k_in, a_transposed=1, b=dy, ldb=n_out,
        b_rowmajor=1, c_f32=part, ldc=n_out, split_stride=k_in * n_out)
    close(part.sum(0), x.float().t() @ dy.float())


def test_rejects_misaligned(wclib, torch):
    a = rnd(torch, 16, 12, seed=1)
    wt = rnd(torch, 16, 12, seed=2)
    c = torch.zeros(16, 16, device="cuda")
    g = _abi.GemmDesc(m=16, n=16, k=12, k_chunk=64, a=a.data_ptr(), lda=12, b=wt.data_ptr(), ldb=12,
                      c_f32=c.data_ptr(), ldc=16)
    assert wclib.wc_nn_gemm(C.byref(g), None, None) == _abi.WC_ERR_INVALID_ARG


@pytest.mark.parametrize("m,n,k", [(58445, 128, 384), (20000, 256, 128)])
def test_persistent_pipeline_many_tiles(wclib, torch, m, n, k):
    """Several output tiles per CTA: the persistent kernel's operand ring wraps around many times
    and both tensor-memory accumulators are reused (their epilogues overlap the next tile's MMAs)."""
    a = rnd(torch, m, k, seed=11)
    wt = rnd(torch, n, k, seed=12)
    bias = torch.randn(n, device="cuda")
    c = torch.zeros(m, n, device="cuda")
    c16 = torch.zeros(m, n, dtype=torch.bfloat16, device="cuda")
    run(wclib, torch, m=m, n=n, k=k, a=a, lda=k, b=wt, ldb=k, bias=bias, relu=1, c_f32=c, c_bf16=c16, ldc=n)
    ref = torch.relu(a.float() @ wt.float().t() + bias)
    close(c, ref)
    close(c16, ref, rel=1e-3 + 2.0 ** -8)


@pytest.mark.parametrize("m,k,bias,resid", [(300, 128, True, True), (77, 256, False, True), (20000, 128, True, False),
                                             (58445, 384, True, True)])
def test_layernorm_epilogue(wclib, torch, m, k, bias, resid):
    """C = LN(A . W^T (+ b)) * gamma + beta (+ resid) in the GEMM's epilogue (the message-passing
    rollout's fused second MLP layers) against the same in FP32 on the BF16 inputs: the row
    statistics in FP32 (a different summation order), then one BF16 rounding of the output."""
    n = 128
    a = rnd(torch, m, k, seed=21)
    wt = rnd(torch, n, k, seed=22)
    b = torch.randn(n, device="cuda") if bias else None
    gamma = torch.rand(n, device="cuda") + 0.5
    beta = torch.randn(n, device="cuda") * 0.1
    r = rnd(torch, m, n, seed=23) if resid else None
    c = torch.zeros(m, n, device="cuda", dtype=torch.bfloat16)
    kw = dict(m=m, n=n, k=k, a=a, lda=k, b=wt, ldb=k, c_bf16=c, ldc=n, ln_gamma=gamma, ln_beta=beta)
    if bias:
        kw["bias"] = b
    if resid:
        kw["ln_resid"] = r
    run(wclib, torch, **kw)
    y = a.float() @ wt.float().t() + (b if bias else 0.0)
    ref = torch.nn.functional.layer_norm(y, (n,), gamma, beta, eps=1e-5) + (r.float() if resid else 0.0)
    close(c, ref, rel=8e-3)


def test_layernorm_epilogue_rejects_other_forms(wclib, torch):
    a = rnd(torch, 64, 64, seed=1)
    wt = rnd(torch, 96, 64, seed=2)
    gamma = torch.ones(96, device="cuda")
    c = torch.zeros(64, 96, device="cuda", dtype=torch.bfloat16)
    g = _abi.GemmDesc(m=64, n=96, k=64, k_chunk=64, a=a.data_ptr(), lda=64, b=wt.data_ptr(), ldb=64,
                      c_bf16=c.data_ptr(), ldc=96, ln_gamma=gamma.data_ptr(), ln_beta=gamma.data_ptr())
    assert wclib.wc_nn_gemm(C.byref(g), None, None) == _abi.WC_ERR_INVALID_ARG  # n must be 128
