"""The MLP's BF16 tensor-core kernels against the numpy oracle, and the learned
initial iterate inside linearized TRT steps (same answers, its own iterations).

Tolerances: GEMM 1e-5 relative to the BF16-rounded operands' float64 product
(FP32 accumulation); gradients 2e-3 relative (FP32 accumulation and BF16
re-rounding of the FP32 intermediate values between the two codes); TRT
temperatures with and without the learned iterate 1e-6 (both solves converge
to 1e-10)."""
import numpy as np
import pytest

from oracle.mlp_oracle import bf16, loss_and_grads

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tc", [True, False])
@pytest.mark.parametrize("M,N,K,ta,tb", [(1, 1, 1, False, False), (70, 33, 45, False, False),
                                         (300, 256, 128, False, False), (45, 70, 33, True, False),
                                         (64, 96, 200, False, True), (129, 65, 300, True, True),
                                         (1000, 384, 712, False, True)])
def test_gemm(M, N, K, ta, tb, tc):
    # tc: the tcgen05 kernel (TMEM accumulator, operands by cp.async.bulk.tensor);
    # else the mma.sync kernel
    from allium_gb300.mlp import gemm, tc_status
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(size=(K, M) if ta else (M, K)).astype(np.float32)
    B = rng.normal(size=(N, K) if tb else (K, N)).astype(np.float32)
    bias = rng.normal(size=N).astype(np.float32)
    C0 = rng.normal(size=(M, N)).astype(np.float32)
    dA = torch.from_numpy(A).cuda().to(torch.bfloat16)
    dB = torch.from_numpy(B).cuda().to(torch.bfloat16)
    out = torch.from_numpy(C0.copy()).cuda()
    gemm(dA, dB, out=out, bias=torch.from_numpy(bias).cuda(), relu=True, alpha=0.5, beta=2.0, transA=ta, transB=tb,
         tc=tc)
    tc_status()
    a = bf16(A).T if ta else bf16(A)
    b = bf16(B).T if tb else bf16(B)
    ref = np.maximum(0.5 * (a @ b) + 2.0 * C0 + bias, 0.0)
    got = out.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-5 * max(1.0, np.max(np.abs(ref)))


def test_gradients_match_oracle():
    from allium_gb300.mlp import CellMLP
    net = CellMLP(37, 11, width=64, layers=4, seed=2)
    rng = np.random.default_rng(4)
    X = rng.normal(size=(257, 37)).astype(np.float32)
    T = rng.normal(size=(257, 11)).astype(np.float32)
    dX, dT = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    Y = net.forward(dX, keep=True)
    dY, loss = net.mse_grad(Y, dT)
    gW, gb = net.backward(dY)
    Ws = [w.cpu().numpy().astype(np.float64) for w in net.W]
    bs = [b.cpu().numpy().astype(np.float64) for b in net.b]
    lo, oW, ob = loss_and_grads(Ws, bs, X, T)
    assert abs(loss.item() - lo) < 1e-4 * lo
    for g, o in zip(gW + gb, oW + ob):
        g = g.cpu().numpy()
        assert np.linalg.norm(g - o) <= 2e-3 * np.linalg.norm(o)


def test_training_reduces_loss():
    from allium_gb300.mlp import CellMLP
    net = CellMLP(8, 4, width=128, layers=4, seed=0, lr=2e-3)
    rng = np.random.default_rng(0)
    X = torch.from_numpy(rng.uniform(-1, 1, size=(2048, 8)).astype(np.float32)).cuda()
    W = torch.from_numpy(rng.normal(size=(8, 4)).astype(np.float32)).cuda()
    T = torch.sin(X @ W)
    first = net.train_step(X, T).item()
    for _ in range(300):
        last = net.train_step(X, T).item()
    assert last < 0.1 * first


def test_learned_iterate_keeps_answers():
    from allium_gb300.mlp import LearnedInitialIterate
    from allium_gb300.trt import marshak_wave
    plain = marshak_wave(cells=16, G=8, tol=1e-10)
    learn = marshak_wave(cells=16, G=8, tol=1e-10)
    li = LearnedInitialIterate(learn, width=64, seed=0)
    for n in range(12):
        plain.step()
        before = (learn.phi(), learn.T.clone(), learn.sigma.clone())
        if n < 8:
            r = learn.step()
            if n > 0:
                li.record(*before, learn.phi())
        else:
            if li.stats is None:
                li.train(epochs=30)
            r = learn.step(phi0=li.predict(*before))
        assert r.converged
        err = torch.max(torch.abs(learn.T - plain.T)).item() / torch.max(plain.T).item()
        assert err < 1e-6


@pytest.mark.parametrize("tc", [True, False])
@pytest.mark.parametrize("M,N,K,ta", [(37, 64, 5000, True), (133, 256, 16384, True), (64, 64, 300, False)])
def test_gemm_split_k(M, N, K, ta, tc):
    # few output tiles over a long K: the kernel splits K over blocks and adds
    # the partial sums atomically (the weight gradients X^T dY over a batch)
    from allium_gb300.mlp import gemm, tc_status
    rng = np.random.default_rng(K)
    A = rng.normal(size=(K, M) if ta else (M, K)).astype(np.float32)
    B = rng.normal(size=(K, N)).astype(np.float32)
    out = gemm(torch.from_numpy(A).cuda().to(torch.bfloat16), torch.from_numpy(B).cuda().to(torch.bfloat16),
               transA=ta, tc=tc)
    tc_status()
    a = bf16(A).T if ta else bf16(A)
    ref = a @ bf16(B)
    assert np.max(np.abs(out.cpu().numpy() - ref)) <= 1e-5 * np.max(np.abs(ref))
