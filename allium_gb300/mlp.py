"""A per-cell MLP trained and evaluated with the library's BF16 tensor-core
kernels (allium_mlp_*: GEMMs with FP32 accumulation and a fused bias / ReLU
epilogue on the fifth-generation tensor cores (tcgen05.mma, TMEM accumulators,
operands by cp.async.bulk.tensor), ReLU/bias/MSE gradients, Adam).  The
warp-level mma.sync GEMM stays available (gemm(..., tc=False)) as the
comparison.

CellMLP is layers x width (ReLU between layers, linear output), FP32 master
weights W_l[K][N] with BF16 copies for the GEMMs.  LearnedInitialIterate wraps
it for a LinearizedTRT calculation: it records (state of step n -> moments of
step n + 1) pairs from plain steps, trains on them, and afterwards predicts the
next step's moments, which become the initial iterate of the step's Schur
solve.  The solve still runs to its tolerance, so a prediction can only change
how many iterations a step takes, never the answer.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _ck(st):
    if st != 0:
        raise _lib.AlliumError(st, _lib.lib().allium_status_string(st).decode())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def to_bf16(x):
    """BF16 copy of an FP32 tensor (allium_mlp_to_bf16)."""
    x = x.contiguous()
    y = torch.empty(x.shape, dtype=torch.bfloat16, device=x.device)
    _ck(_lib.lib().allium_mlp_to_bf16(x.numel(), _p(x), _p(y), _stream()))
    return y


def _kmajor(X, trans):
    """op(X) as a K-major BF16 matrix [R][Kp] with Kp a multiple of 8 (zero
    columns beyond K), as the tensor-core GEMM's tensor maps need: X itself
    when it already is one, else a copy (allium_mlp_transpose_bf16 when the
    operand is stored transposed)."""
    R, K = (X.shape[1], X.shape[0]) if trans else (X.shape[0], X.shape[1])
    Kp = (K + 7) // 8 * 8
    if not trans and Kp == K and X.stride(1) == 1 and X.stride(0) % 8 == 0 and X.data_ptr() % 16 == 0:
        return X, X.stride(0)
    out = (torch.zeros if Kp != K else torch.empty)((R, Kp), dtype=torch.bfloat16, device=X.device)
    if trans:
        assert X.stride(1) == 1
        _ck(_lib.lib().allium_mlp_transpose_bf16(K, R, _p(X), X.stride(0), _p(out), Kp, _stream()))
    else:
        out[:, :K] = X
    return out, Kp


def gemm(A, B, out=None, out_bf16=None, bias=None, relu=False, alpha=1.0, beta=0.0, transA=False, transB=False,
         tc=True):
    """out[M][N] = alpha op(A) op(B) (+ beta out) (+ bias) (ReLU); A, B BF16 2-D tensors.
    tc: the tcgen05 kernel (operands made K-major first where needed), else
    the mma.sync kernel, which reads any strides."""
    M, K = (A.shape[1], A.shape[0]) if transA else (A.shape[0], A.shape[1])
    K2, N = (B.shape[1], B.shape[0]) if transB else (B.shape[0], B.shape[1])
    assert K == K2 and A.dtype == torch.bfloat16 and B.dtype == torch.bfloat16
    if tc:
        return gemm_tc(A, B, out, out_bf16, bias, relu, alpha, beta, transA, transB)
    sam, sak = (1, A.stride(0)) if transA else (A.stride(0), 1)
    sbk, sbn = (1, B.stride(0)) if transB else (B.stride(0), 1)
    assert A.stride(1) == 1 and B.stride(1) == 1
    if out is None and out_bf16 is None:
        out = torch.empty((M, N), dtype=torch.float32, device=A.device)
    ldc = (out if out is not None else out_bf16).stride(0)
    _ck(_lib.lib().allium_mlp_gemm(M, N, K, _p(A), sam, sak, _p(B), sbk, sbn, _p(out), ldc, _p(out_bf16), _p(bias),
                                   float(alpha), float(beta), int(relu), _stream()))
    return out


def gemm_tc(A, B, out=None, out_bf16=None, bias=None, relu=False, alpha=1.0, beta=0.0, transA=False, transB=False):
    """gemm() on the tcgen05 kernel (allium_mlp_gemm_tc: C = A B^T with both
    operands K-major).  Few output tiles over a long K (the weight gradients
    over a batch) split K over blocks, partial sums added atomically."""
    M, K = (A.shape[1], A.shape[0]) if transA else (A.shape[0], A.shape[1])
    N = B.shape[0] if transB else B.shape[1]
    a, lda = _kmajor(A, transA)
    b, ldb = _kmajor(B, not transB)
    if out is None and out_bf16 is None:
        out = torch.empty((M, N), dtype=torch.float32, device=A.device)
    bn = 256 if N > 128 else 128          # the kernel's tile width in N
    tiles = ((M + 127) // 128) * ((N + bn - 1) // bn)
    ksplit = 1
    plain = out is not None and out_bf16 is None and bias is None and not relu and beta == 0.0
    if plain and tiles < 152 and K >= 8 * 64:
        ksplit = max(1, min((152 + tiles - 1) // tiles, K // (4 * 64)))
    ldc = out.stride(0) if out is not None else 0
    ldcb = out_bf16.stride(0) if out_bf16 is not None else 0
    _ck(_lib.lib().allium_mlp_gemm_tc(M, N, K, _p(a), lda, _p(b), ldb, _p(out), ldc,
                                      _p(out_bf16), ldcb, _p(bias), float(alpha), float(beta), int(relu), ksplit,
                                      _stream()))
    return out


def tc_status():
    """Raises if a bounded wait inside the tensor-core GEMM gave up (synchronizes)."""
    _ck(_lib.lib().allium_mlp_status(_stream()))


class CellMLP:
    def __init__(self, n_in, n_out, width=256, layers=4, seed=0, lr=1e-3, device="cuda"):
        g = torch.Generator(device="cpu").manual_seed(seed)
        dims = [n_in] + [width] * (layers - 1) + [n_out]
        self.dims = dims
        self.W, self.b, self.Wb = [], [], []
        self.mW, self.vW, self.mb, self.vb = [], [], [], []
        for k, n in zip(dims[:-1], dims[1:]):
            w = (torch.randn((k, n), generator=g) * math.sqrt(2.0 / k)).to(device=device, dtype=torch.float32)
            self.W.append(w)
            self.Wb.append(w.to(torch.bfloat16))
            self.b.append(torch.zeros(n, dtype=torch.float32, device=device))
            for lst, shape in ((self.mW, (k, n)), (self.vW, (k, n)), (self.mb, (n,)), (self.vb, (n,))):
                lst.append(torch.zeros(shape, dtype=torch.float32, device=device))
        self.lr = lr
        self.step_count = 0

    def forward(self, X, keep=False):
        """X [B][n_in] FP32 -> Y [B][n_out] FP32; keep=True stores activations for backward."""
        h = to_bf16(X)
        acts = [h]
        outs = []
        L = len(self.W)
        for l in range(L):
            last = l == L - 1
            z = torch.empty((X.shape[0], self.dims[l + 1]), dtype=torch.float32, device=X.device)
            hb = None if last else torch.empty_like(z, dtype=torch.bfloat16)
            gemm(h, self.Wb[l], out=z, out_bf16=hb, bias=self.b[l], relu=not last)
            outs.append(z)
            if not last:
                acts.append(hb)
                h = hb
        if keep:
            self._acts, self._outs = acts, outs
        return outs[-1]

    def backward(self, dY):
        """Gradients of the weights for dY = dLoss/dY of the last forward(keep=True)."""
        L = len(self.W)
        B = dY.shape[0]
        lib = _lib.lib()
        gW, gb = [None] * L, [None] * L
        dz = dY.contiguous()
        dzb = to_bf16(dz)
        for l in reversed(range(L)):
            gW[l] = gemm(self._acts[l], dzb, transA=True)                     # H_l^T dZ_l
            gb[l] = torch.empty(self.dims[l + 1], dtype=torch.float32, device=dY.device)
            _ck(lib.allium_mlp_bias_grad(B, self.dims[l + 1], _p(dz), _p(gb[l]), _stream()))
            if l > 0:
                dh = gemm(dzb, self.Wb[l], transB=True)                           # dZ_l W_l^T
                dz = torch.empty_like(dh)
                dzb = torch.empty_like(dh, dtype=torch.bfloat16)
                _ck(lib.allium_mlp_relu_backward(dh.numel(), _p(dh), _p(self._outs[l - 1]), _p(dz), _p(dzb), _stream()))
        return gW, gb

    def mse_grad(self, Y, target):
        count = Y.numel()
        dY = torch.empty_like(Y)
        parts = torch.empty((count + 255) // 256, dtype=torch.float32, device=Y.device)
        _ck(_lib.lib().allium_mlp_mse_grad(count, _p(Y), _p(target.contiguous()), _p(dY), _p(parts), _stream()))
        return dY, parts.sum() / count

    def adam(self, gW, gb, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        lib = _lib.lib()
        for l in range(len(self.W)):
            _ck(lib.allium_mlp_adam(self.W[l].numel(), _p(self.W[l]), _p(self.Wb[l]), _p(gW[l]), _p(self.mW[l]),
                                    _p(self.vW[l]), float(self.lr), b1, b2, eps, self.step_count, _stream()))
            _ck(lib.allium_mlp_adam(self.b[l].numel(), _p(self.b[l]), None, _p(gb[l]), _p(self.mb[l]),
                                    _p(self.vb[l]), float(self.lr), b1, b2, eps, self.step_count, _stream()))

    def train_step(self, X, target):
        Y = self.forward(X, keep=True)
        dY, loss = self.mse_grad(Y, target)
        gW, gb = self.backward(dY)
        self.adam(gW, gb)
        return loss


def face_neighbours(mesh):
    """[Ne][2 dim] neighbour element across each face (-1 on the boundary),
    from shared face vertex sets (quads: edges; hexes: faces)."""
    if mesh.dim == 2:
        faces = [(0, 1), (1, 2), (2, 3), (3, 0)]
    elif mesh.dim == 3:
        faces = [(0, 1, 2, 3), (4, 5, 6, 7), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7)]
    else:
        faces = [(0,), (1,)]
    ne = mesh.num_elements
    owner = {}
    nbr = -np.ones((ne, len(faces)), dtype=np.int64)
    for e in range(ne):
        ev = mesh.elements[e]
        for k, f in enumerate(faces):
            key = tuple(sorted(int(ev[c]) for c in f))
            if key in owner:
                e2, k2 = owner.pop(key)
                nbr[e, k] = e2
                nbr[e2, k2] = e
            else:
                owner[key] = (e, k)
    return nbr


class LearnedInitialIterate:
    """Per-cell MLP predicting the next step's moments of a LinearizedTRT.

    The prediction is the linear extrapolation phi_n + (phi_n - phi_{n-1})
    plus a learned correction.  Input of cell e (standardised): log10 of the
    cell-mean moment of every group, the cell-mean last change of every group
    over the group's largest moment, log10 sigma_g, log10 of the face
    neighbours' mean moment per group, log10 of the cell-mean temperature and
    the temperature's nodal shape T_i / T_mean - 1.  Output: the deviation of
    every (group, DOF) moment from the extrapolation over the group's largest
    moment magnitude (standardised).  The network's last layer starts small,
    so an untrained network returns about the extrapolation."""

    def __init__(self, trt, width=256, layers=4, seed=0, lr=1e-3):
        self.trt = trt
        self.G, self.ne, self.n = trt.G, trt.ne, trt.n
        nb = face_neighbours(trt.L.mesh)
        dev = trt.T.device
        self.nb = torch.from_numpy(np.where(nb < 0, np.arange(self.ne)[:, None], nb)).to(dev)
        self.nin = 4 * self.G + 1 + self.n
        self.nout = self.G * self.n
        self.net = CellMLP(self.nin, self.nout, width=width, layers=layers, seed=seed, lr=lr, device=dev)
        self.net.W[-1].mul_(0.01)
        self.net.Wb[-1] = self.net.W[-1].to(torch.bfloat16)
        self.X, self.Y = [], []
        self.stats = None
        self.losses = []
        self.gain = 1.0
        self.last = None        # moments before the previous step

    def _scale(self, phi):
        return phi.view(self.G, -1).abs().amax(dim=1).clamp(min=1e-300)

    def _step_change(self, phi):
        return phi - self.last if self.last is not None else torch.zeros_like(phi)

    def features(self, phi, dphi, T, sigma):
        G, ne, n = self.G, self.ne, self.n
        pm = phi.view(G, ne, n).mean(dim=2)                          # [G][Ne]
        lp = torch.log10(pm.abs().clamp(min=1e-300))
        dm = dphi.view(G, ne, n).mean(dim=2) / self._scale(phi).view(G, 1)
        ls = torch.log10(sigma.view(G, ne).clamp(min=1e-300))
        nbm = pm[:, self.nb].mean(dim=2)                              # [G][Ne]
        ln = torch.log10(nbm.abs().clamp(min=1e-300))
        Tc = T.view(ne, n)
        Tm = Tc.mean(dim=1, keepdim=True)
        shape = Tc / Tm.clamp(min=1e-300) - 1.0
        X = torch.cat([lp.t(), dm.t(), ls.t(), ln.t(), torch.log10(Tm.clamp(min=1e-300)), shape], dim=1)
        return X.float()

    def target(self, base, phi_new, scale):
        d = (phi_new - base).view(self.G, self.ne, self.n) / scale.view(self.G, 1, 1)
        return d.permute(1, 0, 2).reshape(self.ne, self.G * self.n).float()

    def record(self, phi_old, T_old, sigma_old, phi_new):
        """A training pair: state before a step -> moments after it."""
        d = self._step_change(phi_old)
        self.X.append(self.features(phi_old, d, T_old, sigma_old))
        self.Y.append(self.target(phi_old + d, phi_new, self._scale(phi_old)))
        self.last = phi_old.clone()

    def extrapolate(self, phi):
        """phi_n + (phi_n - phi_{n-1}), the prediction without the network."""
        d = self._step_change(phi)
        self.last = phi.clone()
        return phi + d

    def train(self, epochs=20, holdout=0.1):
        """Train on all but the last `holdout` fraction of the recorded steps;
        on those later steps fit the gain in [0, 1] applied to the network's
        correction (0 when the correction does not beat the extrapolation)."""
        nval = max(1, int(round(holdout * len(self.X)))) if len(self.X) > 1 else 0
        X = torch.cat(self.X[:len(self.X) - nval])
        Y = torch.cat(self.Y[:len(self.Y) - nval])
        mx, sx = X.mean(0), X.std(0).clamp(min=1e-6)
        my, sy = Y.mean(0), Y.std(0).clamp(min=1e-12)
        self.stats = (mx, sx, my, sy)
        Xn, Yn = (X - mx) / sx, (Y - my) / sy
        B = self.ne
        perm_gen = torch.Generator(device="cpu").manual_seed(1)
        for _ in range(epochs):
            order = torch.randperm(Xn.shape[0], generator=perm_gen).to(Xn.device)
            for k in range(0, Xn.shape[0] - B + 1, B):
                idx = order[k:k + B]
                self.losses.append(self.net.train_step(Xn[idx].contiguous(), Yn[idx].contiguous()))
        self.gain = 1.0
        if nval:
            Xv = torch.cat(self.X[len(self.X) - nval:])
            Yv = torch.cat(self.Y[len(self.Y) - nval:]).double()
            pv = (self.net.forward(((Xv - mx) / sx).contiguous()) * sy + my).double()
            den = torch.dot(pv.reshape(-1), pv.reshape(-1)).item()
            a = torch.dot(Yv.reshape(-1), pv.reshape(-1)).item() / den if den > 0 else 0.0
            self.gain = min(1.0, max(0.0, a))
        return float(self.losses[-1].item()) if self.losses else None

    def predict(self, phi, T, sigma):
        mx, sx, my, sy = self.stats
        d = self._step_change(phi)
        Y = self.net.forward(((self.features(phi, d, T, sigma) - mx) / sx).contiguous()) * sy + my
        corr = self.gain * Y.view(self.ne, self.G, self.n).permute(1, 0, 2).reshape(-1).double()
        s = self._scale(phi)
        self.last = phi.clone()
        return phi + d + corr * s.repeat_interleave(self.ne * self.n)
