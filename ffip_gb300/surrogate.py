"""Design-screening surrogate: a small 3-D/2-D convolutional network that maps
a design density to the DFT fields on an output plane, trained on this
project's own GPU FDTD runs.  The reference has no learned part; this is the
rebuild's addition for design loops (a cheap proxy that ranks candidate
design steps, while a full FDTD run checks every accepted step).

Convolutions run on the project's own kernels (libffip_gb300.so,
include/ffip_gb300_surrogate.h): im2col, a bf16 tensor-core GEMM with fp32
accumulation, and col2im for the input gradient.  Weights are kept in fp32
(Adam updates them), cast to bf16 for each GEMM; activations are bf16.

  python -m ffip_gb300.surrogate --designs 2048 --epochs 50 --out result.json

generates the designs, trains, reports the error on held-out FDTD runs and
runs the screened versus plain design loop (see run_study).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import time
from typing import List, Optional

import numpy as np

from . import native

_L = None


def lib():
    """The native library with the surrogate kernels declared."""
    global _L
    if _L is None:
        L = native.load()
        P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        IP = ctypes.POINTER(ctypes.c_int)
        L.ffip_sg_gemm.argtypes = [I, I, I, P, I64, I64, P, I64, I64, P, I64, I64, P, I, P]
        L.ffip_sg_gemm_path.argtypes = [I, I, I, P, I64, I64, P, I64, I64, P, I64, I64, P, I, P, I]
        L.ffip_sg_check.argtypes = []
        L.ffip_sg_im2col.argtypes = [P, IP, IP, IP, IP, P, P]
        L.ffip_sg_im2col_t.argtypes = [P, IP, IP, IP, IP, P, P]
        L.ffip_sg_col2im.argtypes = [P, IP, IP, IP, IP, P, P]
        for f in ("ffip_sg_gemm", "ffip_sg_gemm_path", "ffip_sg_check", "ffip_sg_im2col", "ffip_sg_im2col_t",
                  "ffip_sg_col2im"):
            getattr(L, f).restype = ctypes.c_int
        _L = L
    return _L


def _torch():
    import torch
    return torch


def _check(rc):
    if rc != 0:
        raise native.FfipError(lib().ffip_last_error().decode(errors="replace"))


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def gemm(A, B, bias=None, out=None, accumulate=False, path=0):
    """out[M,N] (fp32) = A[M,K] @ B[K,N] (+ bias), A and B bf16 2-D CUDA
    tensors of any strides (on the project's tensor-core GEMMs: tcgen05 when
    K is contiguous in both, A.stride(1) == 1 and B.stride(0) == 1, mma.sync
    otherwise; path 1 / 2 forces one of them)."""
    torch = _torch()
    if A.dtype != torch.bfloat16 or B.dtype != torch.bfloat16:
        raise TypeError("gemm takes bf16 operands")
    if A.dim() != 2 or B.dim() != 2 or A.shape[1] != B.shape[0]:
        raise ValueError("gemm shapes do not match: %s @ %s" % (tuple(A.shape), tuple(B.shape)))
    M, K = A.shape
    N = B.shape[1]
    if out is None:
        out = torch.empty((M, N), dtype=torch.float32, device=A.device)
        accumulate = False
    if out.dtype != torch.float32 or tuple(out.shape) != (M, N):
        raise ValueError("gemm output must be fp32 of shape (M, N)")
    if bias is not None and (bias.dtype != torch.float32 or not bias.is_contiguous()):
        raise ValueError("bias must be a contiguous fp32 vector")
    _check(lib().ffip_sg_gemm_path(M, N, K, A.data_ptr(), A.stride(0), A.stride(1), B.data_ptr(), B.stride(0), B.stride(1),
                                   out.data_ptr(), out.stride(0), out.stride(1), bias.data_ptr() if bias is not None else None,
                                   1 if accumulate else 0, _stream(), int(path)))
    return out


def check():
    """Synchronises and raises if a tcgen05 GEMM gave up on a bounded wait."""
    _check(lib().ffip_sg_check())


def _ints(v):
    return (ctypes.c_int * len(v))(*[int(x) for x in v])


def conv_out(shape, kernel, stride, pad):
    return tuple((shape[2 + i] + 2 * pad[i] - kernel[i]) // stride[i] + 1 for i in range(3))


def im2col(x, kernel, stride, pad):
    torch = _torch()
    x = x.contiguous()
    N, C = x.shape[:2]
    Do, Ho, Wo = conv_out(x.shape, kernel, stride, pad)
    cols = torch.empty((C * kernel[0] * kernel[1] * kernel[2], N * Do * Ho * Wo), dtype=torch.bfloat16, device=x.device)
    _check(lib().ffip_sg_im2col(x.data_ptr(), _ints(x.shape), _ints(kernel), _ints(stride), _ints(pad), cols.data_ptr(),
                                _stream()))
    return cols


def im2col_t(x, kernel, stride, pad):
    """The column matrix transposed, [N*Do*Ho*Wo, C*kd*kh*kw]: the forward
    GEMM's reduction index contiguous."""
    torch = _torch()
    x = x.contiguous()
    N, C = x.shape[:2]
    Do, Ho, Wo = conv_out(x.shape, kernel, stride, pad)
    colsT = torch.empty((N * Do * Ho * Wo, C * kernel[0] * kernel[1] * kernel[2]), dtype=torch.bfloat16, device=x.device)
    _check(lib().ffip_sg_im2col_t(x.data_ptr(), _ints(x.shape), _ints(kernel), _ints(stride), _ints(pad), colsT.data_ptr(),
                                  _stream()))
    return colsT


def col2im(dcols, shape, kernel, stride, pad):
    torch = _torch()
    dcols = dcols.contiguous()
    dx = torch.empty(tuple(shape), dtype=torch.float32, device=dcols.device)
    _check(lib().ffip_sg_col2im(dcols.data_ptr(), _ints(shape), _ints(kernel), _ints(stride), _ints(pad), dx.data_ptr(),
                                _stream()))
    return dx


_Conv = None


def conv(x, w, b, stride, pad):
    """3-D convolution (2-D as depth 1) on the project's kernels: x bf16
    [N,C,D,H,W], w fp32 [Co,C,kd,kh,kw], b fp32 [Co]; returns bf16
    [N,Co,Do,Ho,Wo].  Differentiable in x, w and b."""
    global _Conv
    torch = _torch()
    if _Conv is None:
        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, x, w, b, stride, pad):
                kernel = tuple(w.shape[2:])
                # every GEMM below takes its operands with the reduction
                # index contiguous (the tcgen05 kernel's layout) where the
                # sizes allow it
                colsT = im2col_t(x, kernel, stride, pad)  # [N*P, C*k]
                Co = w.shape[0]
                wb = w.reshape(Co, -1).to(torch.bfloat16).contiguous()
                y = gemm(wb, colsT.t(), bias=b.contiguous())  # [Co, N*P]
                N = x.shape[0]
                Do, Ho, Wo = conv_out(x.shape, kernel, stride, pad)
                y = y.reshape(Co, N, Do, Ho, Wo).permute(1, 0, 2, 3, 4).contiguous().to(torch.bfloat16)
                ctx.save_for_backward(x, wb)
                ctx.geom = (tuple(x.shape), kernel, stride, pad, tuple(w.shape))
                return y

            @staticmethod
            def backward(ctx, dy):
                x, wb = ctx.saved_tensors
                xshape, kernel, stride, pad, wshape = ctx.geom
                Co = wshape[0]
                dyb = dy.to(torch.bfloat16)
                dy2 = dyb.permute(1, 0, 2, 3, 4).reshape(Co, -1).contiguous()  # [Co, N*P]
                cols = im2col(x, kernel, stride, pad)  # [C*k, N*P]
                dw = gemm(cols, dy2.t()).t().reshape(wshape)  # dW^T [C*k, Co]
                db = dy2.float().sum(1)
                dx = None
                if ctx.needs_input_grad[0]:
                    dy2t = dyb.permute(0, 2, 3, 4, 1).reshape(-1, Co).contiguous()  # [N*P, Co]
                    dcols = gemm(wb.t().contiguous(), dy2t.t())  # [C*k, N*P]
                    dx = col2im(dcols, xshape, kernel, stride, pad).to(torch.bfloat16)
                return dx, dw, db, None, None

        _Conv = _Fn
    return _Conv.apply(x, w, b, tuple(stride), tuple(pad))


def make_net(out_channels: int = 12, width: int = 32, seed: int = 0):
    """The surrogate, a 3-D / 2-D U-Net: a 3-D encoder of four stride-2
    blocks (width, 2, 4, 8 x width channels; two 3x3x3 convolutions each)
    from a 16 x 64 x 64 density down to 8 width x 1 x 4 x 4, and a 2-D decoder
    of four (x2 nearest upsample, concatenation with the encoder features of
    that size folded to 2-D (channels x depth), 3x3 convolution) stages up to
    64 x 64, where the density itself (16 depth channels) joins; a 1x1
    convolution gives out_channels."""
    torch = _torch()
    nn = torch.nn
    F = torch.nn.functional

    class Net(nn.Module):
        def __init__(self):
            super().__init__()
            g = torch.Generator().manual_seed(seed)
            self.enc = nn.ParameterList()
            self.encb = nn.ParameterList()
            c_in, depth = 1, 16
            skip = []  # channels x depth of each encoder stage's output
            for i in range(4):
                c_out = width * (2 ** i)
                for ci in (c_in, c_out):
                    fan = ci * 27
                    self.enc.append(nn.Parameter(torch.randn(c_out, ci, 3, 3, 3, generator=g) * math.sqrt(2.0 / fan)))
                    self.encb.append(nn.Parameter(torch.zeros(c_out)))
                depth //= 2
                skip.append(c_out * depth)
                c_in = c_out
            self.dec = nn.ParameterList()
            self.decb = nn.ParameterList()
            outs = [4 * width, 2 * width, width, width]
            ins = [skip[3] + skip[2], outs[0] + skip[1], outs[1] + skip[0], outs[2] + 16]
            for i in range(4):
                fan = ins[i] * 9
                self.dec.append(nn.Parameter(torch.randn(outs[i], ins[i], 1, 3, 3, generator=g) * math.sqrt(2.0 / fan)))
                self.decb.append(nn.Parameter(torch.zeros(outs[i])))
            self.head = nn.Parameter(torch.randn(out_channels, width, 1, 1, 1, generator=g) * math.sqrt(1.0 / width))
            self.headb = nn.Parameter(torch.zeros(out_channels))

        def forward(self, rho):
            # rho: [N, 16, 64, 64] (z, y, x) in [0, 1]
            x = (rho.unsqueeze(1) * 2 - 1).to(torch.bfloat16)
            feats = []
            for i in range(8):
                st = 2 if i % 2 == 0 else 1
                x = F.relu(conv(x, self.enc[i], self.encb[i], (st, st, st), (1, 1, 1)))
                if i % 2 == 1:
                    N, C, D, H, W = x.shape
                    feats.append(x.reshape(N, C * D, 1, H, W))
            skips = [feats[2], feats[1], feats[0], (rho.unsqueeze(2) * 2 - 1).to(torch.bfloat16)]
            x = feats[3]
            for i in range(4):
                x = F.interpolate(x, scale_factor=(1, 2, 2), mode="nearest")
                x = torch.cat([x, skips[i]], dim=1)
                x = F.relu(conv(x, self.dec[i], self.decb[i], (1, 1, 1), (0, 1, 1)))
            y = conv(x, self.head, self.headb, (1, 1, 1), (0, 0, 0))
            return y.float().squeeze(2)  # [N, out_channels, 64, 64]

    return Net()


# ---------------------------------------------------------------------------
# data: FDTD runs of the surrogate workload


class DesignWorkload:
    """The surrogate workload: a cells x cells x depth box (dx = 1, Courant
    0.5, CPML of `pml` cells), a design region of dz x dn x dn density nodes
    (eps = 1 + 11 rho) centred at the origin, an Ex current sheet below it
    (Gaussian1, f = 0.1), and the complex Ex, Ey DFT fields on a 64 x 64 plane
    of cell centres above it at three frequencies: 12 real channels.  One
    FDTD simulation is kept on the device; each design only replaces the
    density (ffip_set_density)."""

    FREQS = (0.09, 0.1, 0.11)

    def __init__(self, cells=128, depth=96, pml=16, dn=64, dz=16, plane=64, steps=3000, precision="fp32", device=0):
        from . import workloads
        from .geom import Medium, Two_Medium_Box, Vector3
        from .simulation import PML, Simulation, run_until_time
        from .source import Gaussian1, Source
        V = Vector3
        self.dn, self.dz, self.plane = dn, dz, plane
        self.box = Two_Medium_Box(size=V(dn, dn, dz), center=V(0, 0, 0), dim=V(dn, dn, dz), density=np.zeros((dz, dn, dn)),
                                  medium1=Medium(epsilon=12), medium2=Medium(), suffix="surrogate")
        z_lo = -depth / 2 + pml
        self.sim = Simulation(size=V(cells, cells, depth), resolution=1,
                              pmls=[PML(thickness=pml, sigma_max=workloads.sigma_max(3, pml))],
                              sources=[Source(function=Gaussian1(0.1, cutoff=4, start_time=0.0),
                                              center=V(0, 0, float(np.round((z_lo - dz / 2) / 2))),
                                              size=V(cells - 2 * pml, cells - 2 * pml, 0), field_component="Ex")],
                              precision=precision, device=device)
        self.sim.add_geometry(self.box)
        self.z_out = float(np.round((dz / 2 + depth / 2 - pml) / 2))
        self.dfts = [self.sim.add_dft_fields(center=V(0, 0, self.z_out), size=V(plane, plane, 0), frequency=list(self.FREQS),
                                             field_component=c) for c in ("Ex", "Ey")]
        self.stop = run_until_time(steps * 0.5)
        c = (np.arange(plane) - (plane - 1) / 2.0)
        Z, Y, X = np.meshgrid([self.z_out], c, c, indexing="ij")
        self._pts = {f: np.stack([np.full(X.size, f), Z.ravel(), Y.ravel(), X.ravel()], -1) for f in self.FREQS}
        self._adjoint = None
        self._spec = (cells, depth, pml, precision, device, steps)

    def problem(self, spot: int = 8):
        """The adjoint problem of the spot objective F = -(1/2) sum over the
        central spot x spot cell centres of the output plane, both components
        and the three frequencies, of |E|^2 (= -intensity/2): one broadband
        adjoint run for the three frequencies (design.BroadbandAdjoint), the
        design box shared with the forward simulation."""
        if self._adjoint is not None:
            return self._adjoint
        from . import workloads
        from .design import AdjointProblem, BroadbandAdjoint
        from .geom import Medium, Vector3
        from .simulation import PML, Adjoint_Volume, Simulation, field_match_objective
        from .source import Gaussian1
        V = Vector3
        cells, depth, pml, precision, device, steps = self._spec
        adj = Simulation(size=V(cells, cells, depth), resolution=1,
                         pmls=[PML(thickness=pml, sigma_max=workloads.sigma_max(3, pml))], precision=precision,
                         device=device)
        bb = BroadbandAdjoint(adj, self.sim, Gaussian1(0.1, cutoff=4, start_time=0.0), self.FREQS, 0.5)
        for f in self.FREQS:
            bb.source(f, center=V(0, 0, self.z_out), size=V(spot - 1, spot - 1, 0), dim=V(spot, spot, 1),
                      udfs=[field_match_objective(np.zeros((1, spot, spot)), c, weight=-1.0) for c in ("Ex", "Ey")])
            bb.add_volume(Adjoint_Volume(adj, self.sim, frequency=f, center=V(0, 0, 0), size=V(self.dn, self.dn, self.dz),
                                         dim=V(self.dn, self.dn, self.dz), density=self.box.density,
                                         medium1=Medium(epsilon=12), medium2=Medium(), norm=bb.norm(f), geometry=self.box))
        self._adjoint = AdjointProblem(self.sim, [bb], self.stop)
        return self._adjoint

    def fields(self, rho: np.ndarray) -> np.ndarray:
        """FDTD: the 12 x 64 x 64 output (Re, Im of Ex, Ey at each frequency)."""
        self.box.density = np.asarray(rho, dtype=np.float64)
        self.sim.run(self.stop, keep=True)
        return self.last_fields()

    def last_fields(self) -> np.ndarray:
        """The output of the forward simulation's last run (the design loop's
        forward runs leave it there too)."""
        out = []
        for d in self.dfts:
            it = d.get_interpolant(method="linear")
            for f in self.FREQS:
                v = it(self._pts[f]).reshape(self.plane, self.plane)
                out += [v.real, v.imag]
        return np.stack(out).astype(np.float32)

    def release(self):
        self.sim.release()
        if self._adjoint is not None:
            self._adjoint.release()


def random_designs(n, shape=(16, 64, 64), seed=0, sigma=(2.0, 5.0)):
    """Seeded filtered-noise densities, sigma uniform in the given range."""
    from .workloads import filtered_noise
    rng = np.random.default_rng(seed)
    return np.stack([filtered_noise(shape, float(rng.uniform(*sigma)), int(rng.integers(1 << 31))) for _ in range(n)])


def generate(n, seed=0, workload: Optional[DesignWorkload] = None):
    wl = workload or DesignWorkload()
    rho = random_designs(n, (wl.dz, wl.dn, wl.dn), seed)
    t0 = time.perf_counter()
    y = np.stack([wl.fields(r) for r in rho])
    return rho.astype(np.float32), y, time.perf_counter() - t0


def spot_weights(shape, spot=8, weight=0.0):
    """Per-pixel loss weights of an output plane: 1, and 1 + weight in the
    central spot x spot cells (the region the design objective reads),
    normalised to mean 1."""
    w = np.ones(shape[-2:], dtype=np.float32)
    c0, c1 = shape[-2] // 2 - spot // 2, shape[-1] // 2 - spot // 2
    w[c0:c0 + spot, c1:c1 + spot] += weight
    return w / w.mean()


def train(net, rho, y, epochs=50, batch=32, lr=1e-3, seed=0, log=None, spot_weight=0.0):
    """Adam on the mean squared error of the label-normalised outputs
    (spot_weight > 0: the central spot's pixels weigh 1 + spot_weight)."""
    torch = _torch()
    dev = torch.device("cuda")
    net.to(dev)
    scale = float(np.sqrt(np.mean(y ** 2))) or 1.0
    X = torch.tensor(rho, device=dev)
    Y = torch.tensor(y / scale, device=dev)
    W = torch.tensor(spot_weights(y.shape, weight=spot_weight), device=dev)
    opt = torch.optim.Adam(net.parameters(), lr=lr)
    g = np.random.default_rng(seed)
    hist = []
    t0 = time.perf_counter()
    for ep in range(epochs):
        order = g.permutation(len(X))
        tot = 0.0
        for i in range(0, len(order), batch):
            idx = torch.tensor(order[i:i + batch], device=dev)
            loss = torch.mean(W * (net(X[idx]) - Y[idx]) ** 2)
            opt.zero_grad(set_to_none=True)
            loss.backward()
            opt.step()
            tot += float(loss.detach()) * len(idx)
        hist.append(tot / len(order))
        check()  # a tcgen05 GEMM that gave up on a bounded wait fails the epoch
        if log:
            torch.cuda.synchronize()
            log("epoch %d loss %.5f (%.1f s)" % (ep, hist[-1], time.perf_counter() - t0))
    torch.cuda.synchronize()
    return {"scale": scale, "loss": hist, "seconds": time.perf_counter() - t0}


def predict(net, rho, scale, batch=64):
    torch = _torch()
    dev = torch.device("cuda")
    out = []
    with torch.no_grad():
        for i in range(0, len(rho), batch):
            out.append(net(torch.tensor(np.asarray(rho[i:i + batch], dtype=np.float32), device=dev)).cpu().numpy() * scale)
    check()
    return np.concatenate(out)


def relative_error(pred, y):
    """Per design ||pred - y|| / ||y|| over all 12 channels; mean and max."""
    e = np.sqrt(((pred - y) ** 2).reshape(len(y), -1).sum(1) / (y ** 2).reshape(len(y), -1).sum(1))
    return float(e.mean()), float(e.max())


def spot_objective(fields: np.ndarray, spot: int = 8) -> float:
    """-(1/2) intensity: the adjoint problem's objective (to minimise)."""
    return -0.5 * intensity(fields, spot)


def intensity(fields: np.ndarray, spot: int = 8) -> float:
    """Design objective on the output plane: |Ex|^2 + |Ey|^2 summed over the
    central spot x spot cells and the three frequencies (to maximise)."""
    c0 = fields.shape[-1] // 2 - spot // 2
    f = fields[..., c0:c0 + spot, c0:c0 + spot]
    return float((f ** 2).sum())


class OnlineRefiner:
    """Refines the surrogate on the design loop's own FDTD runs: every
    forward run of a screened candidate adds (design, output fields) to a
    buffer, and `steps` Adam steps on the buffer's latest `window` samples
    (together with as many samples of the training set) follow, so that the
    network learns the neighbourhood the loop moves through."""

    def __init__(self, net, wl, scale, train_rho, train_y, steps=8, window=16, lr=1e-3, seed=0, spot_weight=0.0):
        torch = _torch()
        self.net, self.wl, self.scale, self.steps, self.window = net, wl, scale, steps, window
        self.W = torch.tensor(spot_weights(train_y.shape, weight=spot_weight), device=torch.device("cuda"))
        self.rho, self.y = train_rho, train_y
        self.opt = torch.optim.Adam(net.parameters(), lr=lr)
        self.buf_x, self.buf_y = [], []
        self.rng = np.random.default_rng(seed)
        self.seconds = 0.0

    def __call__(self, x):
        torch = _torch()
        t0 = time.perf_counter()
        self.buf_x.append(np.asarray(x, dtype=np.float32))
        self.buf_y.append(self.wl.last_fields() / self.scale)
        dev = torch.device("cuda")
        bx = np.stack(self.buf_x[-self.window:])
        by = np.stack(self.buf_y[-self.window:])
        for _ in range(self.steps):
            idx = self.rng.integers(0, len(self.rho), size=len(bx))
            X = torch.tensor(np.concatenate([bx, self.rho[idx]]), device=dev)
            Y = torch.tensor(np.concatenate([by, self.y[idx] / self.scale]), device=dev)
            loss = torch.mean(self.W * (self.net(X) - Y) ** 2)
            self.opt.zero_grad(set_to_none=True)
            loss.backward()
            self.opt.step()
        torch.cuda.synchronize()
        self.seconds += time.perf_counter() - t0


def design_loop(prob, x0, steps, mode, net=None, scale=1.0, max_accepted=8, target=None, max_iters=None, rng=None,
                observe=None):
    """Minimise the problem's objective from x0 along its adjoint gradient
    (one forward and one broadband adjoint run per gradient), trying the
    step sizes `steps` along the normalised steepest-descent direction:
      plain:    every step size checked by a forward FDTD run, the best kept;
      screened: the surrogate `net` ranks the step sizes and forward runs
                check the best two in turn (mode "random": the same with a
                random order, the loop without a model).
    Every accepted step is an FDTD-verified improvement.  Stops after
    `max_accepted` accepted steps, or once the objective is at or below
    `target`.  observe(x): called after each screened candidate's forward
    run (an OnlineRefiner).  Returns seconds, FDTD runs and the objective
    trace."""
    x = np.asarray(x0, dtype=np.float64).copy()
    steps = np.asarray(steps, dtype=np.float64)
    max_iters = max_iters or 3 * max_accepted
    t0 = time.perf_counter()
    F, g = prob.value_and_gradient(x)
    runs = 1 + len(prob.terms)
    accepted, trace, runs_at = 0, [F], [runs]
    for _ in range(max_iters):
        if accepted >= max_accepted or (target is not None and F <= target):
            break
        d = -g / max(np.abs(g).max(), 1e-30)
        cands = [np.clip(x + s_ * d, 0, 1) for s_ in steps]
        if mode == "plain":
            vals = [prob.forward(c) for c in cands]
            runs += len(cands)
            best = int(np.argmin(vals))
            if vals[best] < F:
                x = cands[best]
                F, g = prob.value_and_gradient(x)
                runs += 1 + len(prob.terms)
                accepted += 1
                trace.append(F)
                runs_at.append(runs)
            else:
                steps = steps / 4
            continue
        if mode == "screened":
            pred = predict(net, np.stack(cands).astype(np.float32), scale)
            order = np.argsort([spot_objective(q) for q in pred])
        else:
            order = (rng or np.random.default_rng(0)).permutation(len(cands))
        ok = False
        for j in order[:2]:
            v = prob.forward(cands[j])
            runs += 1
            if observe is not None:
                observe(cands[j])
            if v < F:
                x, F = cands[j], v
                g = prob.gradient()
                runs += len(prob.terms)
                accepted += 1
                trace.append(F)
                runs_at.append(runs)
                ok = True
                break
        if not ok:
            steps = steps / 4
    dt = time.perf_counter() - t0
    return {"accepted": accepted, "seconds": dt, "fdtd_runs": runs, "seconds_per_accepted": dt / max(accepted, 1),
            "objective": trace, "runs_at_accepted": runs_at, "reached": target is None or F <= target}


def compare_loops(wl, net, scale, iters=8, candidates=8, seed=0, log=None, train_rho=None, train_y=None, spot_weight=0.0):
    """Plain loop for `iters` accepted steps; its final objective is the
    target of the screened loop (trained network; refined online on the
    loop's own runs when the training set is given) and of the same loop
    with a random ranking (no model), each allowed up to 4 x iters accepted
    steps: FDTD runs and seconds to reach an equal objective."""
    import copy
    prob = wl.problem()
    x0 = random_designs(1, (wl.dz, wl.dn, wl.dn), seed + 7)[0]
    steps = np.geomspace(0.01, 0.3, candidates)
    res = {"plain": design_loop(prob, x0, steps, "plain", max_accepted=iters)}
    target = res["plain"]["objective"][-1]
    res["screened"] = design_loop(prob, x0, steps, "screened", net, scale, max_accepted=4 * iters, target=target,
                                  max_iters=12 * iters)
    if train_rho is not None:
        net2 = copy.deepcopy(net)
        ref = OnlineRefiner(net2, wl, scale, train_rho, train_y, seed=seed, spot_weight=spot_weight)
        res["screened_online"] = design_loop(prob, x0, steps, "screened", net2, scale, max_accepted=4 * iters, target=target,
                                             max_iters=12 * iters, observe=ref)
        res["screened_online"]["refine_seconds"] = ref.seconds
    res["random"] = design_loop(prob, x0, steps, "random", max_accepted=4 * iters, target=target, max_iters=12 * iters,
                                rng=np.random.default_rng(seed))
    if log:
        for k, r in res.items():
            log("%s: %d accepted in %.1f s (%d FDTD runs), objective %.5g -> %.5g%s" % (
                k, r["accepted"], r["seconds"], r["fdtd_runs"], r["objective"][0], r["objective"][-1],
                "" if r["reached"] else " (target not reached)"))
    return res


def run_study(designs=2048, held_out=256, epochs=50, iters=8, candidates=8, seed=0, log=print):
    """Generate, train, evaluate on held-out runs, then compare the design
    loops (compare_loops): seconds and FDTD runs to reach the plain loop's
    objective after `iters` accepted steps."""
    wl = DesignWorkload()
    rho, y, t_gen = generate(designs, seed, wl)
    log("generated %d designs in %.1f s" % (designs, t_gen))
    ntr = designs - held_out
    net = make_net(out_channels=y.shape[1], seed=seed)
    nparams = sum(p.numel() for p in net.parameters())
    tr = train(net, rho[:ntr], y[:ntr], epochs=epochs, seed=seed, log=log)
    pred = predict(net, rho[ntr:], tr["scale"])
    err_mean, err_max = relative_error(pred, y[ntr:])
    log("held-out relative error mean %.4f max %.4f" % (err_mean, err_max))
    res = compare_loops(wl, net, tr["scale"], iters, candidates, seed, log, rho[:ntr], y[:ntr])
    wl.release()
    out = {"designs": designs, "held_out": held_out, "generation_seconds": t_gen, "params": nparams,
           "train": {"epochs": epochs, "seconds": tr["seconds"], "final_loss": tr["loss"][-1]},
           "held_out_rel_error_mean": err_mean, "held_out_rel_error_max": err_max, "loops": res}
    if res["screened"]["reached"]:
        out["screened_speedup_equal_objective"] = res["plain"]["seconds"] / res["screened"]["seconds"]
        out["screened_runs_ratio_equal_objective"] = res["plain"]["fdtd_runs"] / res["screened"]["fdtd_runs"]
    if res["random"]["reached"]:
        out["random_speedup_equal_objective"] = res["plain"]["seconds"] / res["random"]["seconds"]
    if res.get("screened_online", {}).get("reached"):
        out["screened_online_runs_ratio_equal_objective"] = res["plain"]["fdtd_runs"] / res["screened_online"]["fdtd_runs"]
    return out


def gemm_bench(M=256, N=32768, K=864, reps=20, log=print):
    """Times both GEMM kernels on one of the network's convolution shapes
    (K-contiguous operands): 5 warm-up calls, `reps` timed with CUDA events;
    returns {path: (ms, TFLOP/s)}."""
    torch = _torch()
    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    Bt = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    out = torch.empty(M, N, device="cuda")
    res = {}
    for path, name in ((1, "tcgen05"), (2, "mma.sync")):
        for _ in range(5):
            gemm(A, Bt.t(), out=out, path=path)
        check()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            gemm(A, Bt.t(), out=out, path=path)
        e1.record()
        torch.cuda.synchronize()
        check()
        ms = e0.elapsed_time(e1) / reps
        res[name] = (ms, 2.0 * M * N * K / ms / 1e9)
        if log:
            log("%s gemm %dx%dx%d: %.4f ms, %.1f TFLOP/s" % (name, M, N, K, ms, res[name][1]))
    return res


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gemm-bench", action="store_true", help="time the two GEMM kernels on a convolution shape")
    ap.add_argument("--designs", type=int, default=2048)
    ap.add_argument("--held-out", type=int, default=256)
    ap.add_argument("--epochs", type=int, default=50)
    ap.add_argument("--iters", type=int, default=8)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    if a.gemm_bench:
        gemm_bench()
        return
    r = run_study(a.designs, a.held_out, a.epochs, a.iters, seed=a.seed)
    txt = json.dumps(r)
    print(txt)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt)


if __name__ == "__main__":
    main()
