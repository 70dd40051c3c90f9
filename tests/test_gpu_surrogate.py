"""The surrogate's kernels (tensor-core bf16 GEMM, im2col, col2im) and its
convolution, forward and backward, against CPU fp64 oracles (numpy / torch on
the CPU in float64) of the same operations on the same bf16-rounded inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _bf(t):
    return t.to(torch.bfloat16)


@pytest.mark.parametrize("M,N,K", [(64, 64, 32), (37, 129, 70), (1, 5, 3), (256, 512, 6912), (32, 4099, 27)])
def test_gemm_matches_fp32_reference(M, N, K):
    from ffip_gb300 import surrogate as S
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N)
    A = _bf(torch.randn(M, K, device="cuda", generator=g))
    B = _bf(torch.randn(K, N, device="cuda", generator=g))
    ref = A.cpu().double().numpy() @ B.cpu().double().numpy()  # CPU fp64 oracle
    got = S.gemm(A, B).cpu().double().numpy()
    # bf16 products are exact in fp32; the fp32 accumulation rounds
    tol = 1e-5 * K ** 0.5 * np.abs(ref).max() + 1e-6
    assert np.abs(got - ref).max() <= tol


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (37, 129, 72), (5, 7, 8), (200, 300, 136), (256, 512, 6912),
                                   (300, 1000, 864)])
def test_tcgen05_and_mma_sync_gemms_match_the_cpu_oracle(M, N, K):
    """Both tensor-core kernels on K-contiguous operands (the tcgen05 layout:
    A[m][k] row-major, B given as B^T[n][k]), with bias, then accumulating
    into the result, against a CPU fp64 oracle."""
    from ffip_gb300 import surrogate as S
    g = torch.Generator(device="cuda").manual_seed(M + 3 * N + 7 * K)
    A = _bf(torch.randn(M, K, device="cuda", generator=g))
    Bt = _bf(torch.randn(N, K, device="cuda", generator=g))
    bias = torch.randn(M, device="cuda", generator=g)
    D = lambda t: t.cpu().double().numpy()  # noqa: E731
    ref = D(A) @ D(Bt).T + D(bias)[:, None]
    tol = 1e-5 * K ** 0.5 * np.abs(ref).max() + 1e-6
    for path in (1, 2):
        out = S.gemm(A, Bt.t(), bias=bias, path=path)
        S.gemm(A, Bt.t(), out=out, accumulate=True, path=path)
        S.check()
        assert np.abs(D(out) - (2 * ref - D(bias)[:, None])).max() <= 2 * tol, path
        assert np.abs(D(S.gemm(A, Bt.t(), bias=bias, path=path)) - ref).max() <= tol, path


def test_tcgen05_gemm_rejects_operands_it_does_not_take():
    from ffip_gb300 import surrogate as S
    A = _bf(torch.randn(16, 24, device="cuda"))
    B = _bf(torch.randn(24, 16, device="cuda"))  # row-major B: k is not contiguous
    with pytest.raises(Exception, match="tensor-core GEMM"):
        S.gemm(A, B, path=1)


def test_gemm_strides_bias_and_accumulate():
    from ffip_gb300 import surrogate as S
    g = torch.Generator(device="cuda").manual_seed(1)
    A = _bf(torch.randn(50, 40, device="cuda", generator=g))       # used transposed: [40, 50]
    B = _bf(torch.randn(90, 50, device="cuda", generator=g)).t()   # [50, 90], column-major view
    bias = torch.randn(40, device="cuda", generator=g)
    C0 = torch.randn(40, 90, device="cuda", generator=g)
    D = lambda t: t.cpu().double().numpy()  # noqa: E731
    ref = D(C0) + (D(A.t()) @ D(B) + D(bias)[:, None])  # CPU fp64 oracle
    out = C0.clone()
    S.gemm(A.t(), B, bias=bias, out=out, accumulate=True)
    assert np.abs(D(out) - ref).max() <= 1e-4


@pytest.mark.parametrize("dims", [3, 2])
def test_conv_forward_and_backward_match_fp32_reference(dims):
    from ffip_gb300 import surrogate as S
    F = torch.nn.functional
    g = torch.Generator(device="cuda").manual_seed(dims)
    if dims == 3:
        x = _bf(torch.randn(3, 5, 6, 10, 9, device="cuda", generator=g))
        w = _bf(torch.randn(7, 5, 3, 3, 3, device="cuda", generator=g) * 0.2).float()
        stride, pad = (2, 2, 2), (1, 1, 1)
    else:
        x = _bf(torch.randn(3, 5, 1, 12, 11, device="cuda", generator=g))
        w = _bf(torch.randn(7, 5, 1, 3, 3, device="cuda", generator=g) * 0.2).float()
        stride, pad = (1, 1, 1), (0, 1, 1)
    b = torch.randn(7, device="cuda", generator=g)
    # CPU fp64 oracle of the convolution and its gradients
    xr = x.cpu().double().requires_grad_(True)
    wr = w.cpu().double().requires_grad_(True)
    br = b.cpu().double().requires_grad_(True)
    yr = F.conv3d(xr, wr, br, stride=stride, padding=pad)
    dy = _bf(torch.randn(yr.shape, device="cuda", generator=g))
    yr.backward(dy.cpu().double())
    xs = x.clone().requires_grad_(True)
    ws = w.clone().requires_grad_(True)
    bs = b.clone().requires_grad_(True)
    ys = S.conv(xs, ws, bs, stride, pad)
    assert ys.dtype == torch.bfloat16 and ys.shape == yr.shape
    C = lambda t: t.detach().cpu().double()  # noqa: E731
    # the forward output is rounded to bf16 (relative 2^-8)
    assert (C(ys) - C(yr)).abs().max().item() <= 1e-2 * C(yr).abs().max().item()
    ys.backward(dy)
    # weight / bias gradients accumulate in fp32 from bf16 operands
    assert (C(ws.grad) - C(wr.grad)).abs().max().item() <= 1e-4 * C(wr.grad).abs().max().item()
    assert (C(bs.grad) - C(br.grad)).abs().max().item() <= 1e-4 * C(br.grad).abs().max().item()
    # the input gradient is rounded to bf16
    assert (C(xs.grad) - C(xr.grad)).abs().max().item() <= 1e-2 * C(xr.grad).abs().max().item()


def test_network_shapes_and_a_few_training_steps_reduce_the_loss():
    from ffip_gb300 import surrogate as S
    net = S.make_net(out_channels=12, width=8, seed=0).cuda()
    rng = np.random.default_rng(0)
    rho = rng.uniform(0, 1, size=(8, 16, 64, 64)).astype(np.float32)
    y = rng.normal(size=(8, 12, 64, 64)).astype(np.float32) * 0.1 + rho[:, :1, ::1, :].mean(1, keepdims=True)[:, :, :64, :64]
    out = net(torch.tensor(rho, device="cuda"))
    assert tuple(out.shape) == (8, 12, 64, 64)
    h = S.train(net, rho, y, epochs=6, batch=4, lr=3e-3)
    assert h["loss"][-1] < h["loss"][0]


def test_screened_loop_reaches_the_plain_loops_objective_with_fewer_fdtd_runs():
    """What the network gains over the loop without it: on a small kept FDTD
    workload (96 x 96 x 64 cells, the surrogate's 64 x 64 x 16 design region
    and 64 x 64 output plane, 1500 steps), a network trained on 288
    FDTD-generated designs (width 8, 30 epochs) and refined online on the
    loop's own forward runs screens the step sizes along the adjoint
    gradient; it reaches the objective that the plain loop (every step size
    checked by a forward run) reaches after 3 accepted steps, with fewer FDTD
    runs.  Every accepted step of both loops is an FDTD-verified
    improvement."""
    from ffip_gb300 import surrogate as S
    wl = S.DesignWorkload(cells=96, depth=64, pml=8, dn=64, dz=16, plane=64, steps=1500)
    try:
        rho, y, _ = S.generate(320, seed=3, workload=wl)
        net = S.make_net(out_channels=y.shape[1], width=8, seed=0)
        tr = S.train(net, rho[:288], y[:288], epochs=30, batch=16, lr=3e-3)
        assert tr["loss"][-1] < tr["loss"][0]
        res = S.compare_loops(wl, net, tr["scale"], iters=3, candidates=8, seed=1, train_rho=rho[:288], train_y=y[:288])
    finally:
        wl.release()
    plain, screened = res["plain"], res["screened_online"]
    assert plain["accepted"] == 3
    assert all(b < a for a, b in zip(plain["objective"], plain["objective"][1:]))
    assert all(b < a for a, b in zip(screened["objective"], screened["objective"][1:]))
    assert screened["reached"], screened["objective"]
    assert screened["fdtd_runs"] < plain["fdtd_runs"], (screened["fdtd_runs"], plain["fdtd_runs"])
