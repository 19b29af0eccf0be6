"""Tensor-core GEMM of the surrogate (tcgen05, bf16 in, fp32 accumulate)
against a plain PyTorch fp32 product of the same bf16 inputs."""

import pytest

torch = pytest.importorskip("torch")

from floodgb import native  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    from floodgb.build import build_library

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")


def bf16(*shape, scale=1.0, seed=0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return (torch.randn(*shape, device="cuda", generator=g) * scale).to(torch.bfloat16)


def close(got, ref, rtol=2e-3):
    err = (got - ref).abs().max().item()
    tol = rtol * max(ref.abs().max().item(), 1.0)
    assert err <= tol, f"max error {err:.3e} > {tol:.3e}"


@pytest.mark.parametrize("tiled", [False, True])
@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (1000, 128, 384), (300, 256, 128), (77, 384, 192),
                                   (40000, 128, 512), (129, 64, 256)])
def test_gemm_plain(m, n, k, tiled):
    from floodgb.surrogate import ops

    a = bf16(m, k, seed=1)
    b = bf16(n, k, scale=0.1, seed=2)
    out = torch.empty(m, n, device="cuda", dtype=torch.float32)
    ops.gemm([(a, None, k)], b, out_f32=out, force_tiled=tiled)
    ops.status()
    close(out, a.float() @ b.float().T)


@pytest.mark.parametrize("tiled", [False, True])
def test_gemm_gathered_segments_bias_relu_residual(tiled):
    from floodgb.surrogate import ops

    nodes, edges, h = 500, 1700, 128
    x = bf16(nodes, h, seed=3)
    e = bf16(edges, h, seed=4)
    g = torch.Generator(device="cuda").manual_seed(5)
    dst = torch.randint(0, nodes, (edges,), device="cuda", generator=g, dtype=torch.int32)
    src = torch.randint(0, nodes, (edges,), device="cuda", generator=g, dtype=torch.int32)
    w = bf16(h, 3 * h, scale=0.05, seed=6)
    bias = torch.randn(h, device="cuda", generator=g)
    res = torch.randn(edges, h, device="cuda", generator=g)
    out = torch.empty(edges, h, device="cuda", dtype=torch.float32)
    outb = torch.empty(edges, h, device="cuda", dtype=torch.bfloat16)
    ops.gemm([(x, dst, h), (x, src, h), (e, None, h)], w, bias=bias, residual=res, out_f32=out, out_bf16=outb,
             relu=True, force_tiled=tiled)
    ops.status()
    cat = torch.cat([x[dst.long()], x[src.long()], e], dim=1).float()
    ref = torch.relu(cat @ w.float().T + bias) + res
    close(out, ref)
    close(outb.float(), ref, rtol=1e-2)


@pytest.mark.parametrize("n", [128, 200])
def test_gemm_epilogue_on_16_byte_aligned_and_padded_outputs(n):
    """Outputs with a leading dimension that is not a multiple of 16 and a
    bias / residual that are 16- but not 32-byte aligned take the epilogue's
    16-byte path; n = 200 also leaves a ragged last 16-column group."""

    from floodgb.surrogate import ops

    m, k, ldo = 700, 128, n + 8
    a = bf16(m, k, seed=7)
    w = bf16(n, k, scale=0.05, seed=8)
    g = torch.Generator(device="cuda").manual_seed(9)
    bias_buf = torch.randn(n + 4, device="cuda", generator=g)
    bias = bias_buf[4:]  # 16-byte offset
    res_buf = torch.randn(m * ldo + 4, device="cuda", generator=g)
    res = res_buf[4:].view(m, ldo)
    outb_buf = torch.zeros(m, ldo, device="cuda", dtype=torch.bfloat16)
    out_buf = torch.zeros(m, ldo, device="cuda", dtype=torch.float32)
    ops.gemm([(a, None, k)], w, bias=bias, residual=res, out_f32=out_buf, out_bf16=outb_buf, relu=True)
    ops.status()
    ref = torch.relu(a.float() @ w.float().T + bias) + res[:, :n]
    close(out_buf[:, :n], ref)
    close(outb_buf[:, :n].float(), ref, rtol=1e-2)
    assert out_buf[:, n:].abs().max().item() == 0.0  # padding columns untouched


def test_gemm_split_k_partials_sum_to_product():
    from floodgb.surrogate import ops

    m, n, k, splits = 256, 128, 1024, 3
    a = bf16(m, k, seed=7)
    b = bf16(n, k, scale=0.05, seed=8)
    part = torch.empty(splits, m, n, device="cuda", dtype=torch.float32)
    ops.gemm([(a, None, k)], b, out_f32=part, k_splits=splits)
    ops.status()
    close(part.sum(0), a.float() @ b.float().T)
