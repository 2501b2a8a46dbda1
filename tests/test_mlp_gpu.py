"""Tensor-core (tcgen05) matrix products of the move-ordering network
against an FP32 reference of the same operands.  Tolerances: BF16 and
E4M3 operands are exactly representable in FP32 and products are exact, so
the only difference is the summation order of FP32 accumulation:
relative error <= 1e-4 of the row's absolute sum."""
import pytest

pytestmark = pytest.mark.gpu


def _check(torch, c, ref):
    scale = ref.abs().max().clamp_min(1.0)
    err = (c - ref).abs().max() / scale
    assert err < 1e-4, float(err)


@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (128, 128, 128), (256, 512, 768), (200, 128, 256),
                                   (384, 256, 512), (64, 16, 64), (512, 768, 128)])
def test_gemm_bf16_matches_fp32(zeta_device, m, n, k):
    torch = pytest.importorskip("torch")
    z = zeta_device
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n * 3 + k)
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    c = torch.full((m, n), float("nan"), device="cuda")
    z.gemm_tc(a.data_ptr(), b.data_ptr(), c.data_ptr(), m, n, k)
    torch.cuda.synchronize()
    ref = a.float() @ b.float().T
    _check(torch, c, ref)


def _dataset(seed, n):
    import numpy as np
    import oracle_lib as ol
    boards, stm, _ = ol.make_positions(seed, n, min_plies=8, max_plies=70, min_pieces=0, min_depth=0, max_depth=0)
    rng = np.random.default_rng(seed)
    targets = np.array([rng.choice(ol.genmoves(boards[i], stm[i])) for i in range(n)], dtype=np.uint32)
    return boards, stm, targets


def test_gradients_match_fp32_oracle(zeta_device):
    """Full backward pass of the network (five tensor-core GEMMs, the loss
    head, bias sums) against the FP32 NumPy oracle.  The kernels keep
    activations in BF16 (8-bit mantissa), so each gradient tensor must
    agree to a relative L2 error below 3e-2 and a cosine above 0.999."""
    import numpy as np
    import mlp_oracle as mo
    z = zeta_device
    z.mlp_init(7)
    boards, stm, targets = _dataset(0x6AD, 256)
    g, loss = z.mlp_grads(boards, stm, targets)
    p = z.mlp_get_params()
    ref_loss, G = mo.loss_and_grads(p, boards, stm, targets)
    assert abs(loss - ref_loss) < 2e-2 * max(1.0, abs(ref_loss))
    got = mo.unflatten(g)
    for name, _ in mo.SHAPES:
        a, b = got[name].ravel().astype(np.float64), G[name].ravel().astype(np.float64)
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
        assert rel < 3e-2 and cos > 0.999, (name, rel, cos)


def test_training_lowers_loss_and_fp8_agrees(zeta_device):
    import numpy as np
    z = zeta_device
    z.mlp_init(11)
    w = z.WORKLOADS["search_batch"]
    boards, stm, _ = z.make_positions(0x7EA, 4096, 10, 60, 0, 0, 0)
    z.tt_clear()
    _, best, _ = z.search_batch(boards, stm, 3, 4)
    loss, acc = z.mlp_train(boards, stm, best, epochs=6, batch=1024, lr=2e-3)
    assert loss[-1] < loss[0] * 0.8, loss
    assert acc[-1] > 0.15, acc  # uniform guessing over ~30 moves is ~0.03
    sb, nb, bb = z.mlp_scores(boards[:512], stm[:512], fp8=False)
    s8, n8, b8 = z.mlp_scores(boards[:512], stm[:512], fp8=True)
    assert np.array_equal(nb, n8)
    assert (bb == b8).mean() > 0.85


@pytest.mark.parametrize("m,n,k", [(128, 64, 128), (256, 256, 512), (130, 128, 768)])
def test_gemm_fp8_matches_fp32(zeta_device, m, n, k):
    torch = pytest.importorskip("torch")
    z = zeta_device
    g = torch.Generator(device="cuda").manual_seed(m + n + k)
    a = (torch.randn(m, k, device="cuda", generator=g) * 2).to(torch.float8_e4m3fn)
    b = (torch.randn(n, k, device="cuda", generator=g) * 2).to(torch.float8_e4m3fn)
    c = torch.full((m, n), float("nan"), device="cuda")
    z.gemm_tc(a.data_ptr(), b.data_ptr(), c.data_ptr(), m, n, k, fp8=True)
    torch.cuda.synchronize()
    ref = a.float() @ b.float().T
    _check(torch, c, ref)


@pytest.mark.parametrize("m,n,k,fp8", [(65536, 512, 768, False), (20000, 384, 256, False), (65536, 256, 512, True),
                                       (40000, 48, 128, False)])
def test_persistent_gemm_many_tiles_per_cta(zeta_device, m, n, k, fp8):
    """Shapes with many more output tiles than SMs, so that every CTA of
    the persistent kernel runs several tiles through both tensor-memory
    accumulators and its ring of K slices runs on from tile to tile (M and
    N not multiples of the tile for two of them).  Against FP32, and bit
    for bit against the per-tile kernel (the same MMAs per tile in the
    same order)."""
    torch = pytest.importorskip("torch")
    z = zeta_device
    g = torch.Generator(device="cuda").manual_seed(m + 3 * n + 7 * k)
    dt = torch.float8_e4m3fn if fp8 else torch.bfloat16
    a = torch.randn(m, k, device="cuda", generator=g).to(dt)
    b = torch.randn(n, k, device="cuda", generator=g).to(dt)
    out = {}
    try:
        for mode in (3, 1):
            z.gemm_configure(mode)
            c = torch.full((m, n), float("nan"), device="cuda")
            z.gemm_tc(a.data_ptr(), b.data_ptr(), c.data_ptr(), m, n, k, fp8=fp8)
            torch.cuda.synchronize()
            out[mode] = c
    finally:
        z.gemm_configure(0)
    _check(torch, out[3], a.float() @ b.float().T)
    assert torch.equal(out[3], out[1])
