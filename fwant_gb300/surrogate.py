"""Learned waveform surrogate for screening line-search candidates.

A small 3-D convolutional network maps a perturbation of the reference model, together
with a feature of the reference wavefield, to the receiver waveforms of the perturbed
model.  It runs entirely on the kernels of ``include/fwant_surrogate.h`` (BF16 weights,
FP32 biases, activations and accumulation, Adam on FP32 master weights); PyTorch only provides
device memory and the stream.  The finite-difference solver is the surrogate's fallback
and the judge of its error: an ensemble of networks estimates the error of each
prediction, and candidates whose estimate exceeds the tolerance are solved by FD.

Network (sizes for the 128x128x64 configuration):
  input  (2, 32, 32, 16): dVs/Vs pooled over 4x4x4 cells (x20), log reference energy
  conv0  2 -> 16, stride 1;  conv1 16 -> 32, stride 2;  conv2 32 -> 32, stride 2
  fc0    32*8*8*4 -> 256;    fc1 256 -> 3 x nsamp x nrecv (the waveform residual)
  leaky ReLU (slope 0.1) after every layer but the last
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._lib import FwantError, load_library

SLOPE = 0.1


def _lib():
    return load_library()


def _ok(rc, what):
    if rc != 0:
        raise FwantError(3, f"{what}: CUDA error {rc}")


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class Net:
    """The surrogate network on one GPU.  convs: [(cin, cout, stride)], dense: [(in, out)],
    in_shape: (C, D, H, W) of one input sample."""

    def __init__(self, in_shape, convs, dense, seed=0, device="cuda", basis=None):
        import torch
        self.torch = torch
        # optional fixed output basis (G, K, T): the dense output is G*K coefficients
        self.basis = basis
        if basis is not None:
            self.G, self.K, self.T = (int(v) for v in basis.shape)
            assert dense[-1][1] == self.G * self.K
        self.L = _lib()
        self.in_shape = tuple(int(v) for v in in_shape)
        self.convs = [tuple(int(v) for v in c) for c in convs]
        self.dense = [tuple(int(v) for v in d) for d in dense]
        self.device = device
        # layer shapes: conv outputs
        shapes = [self.in_shape]
        for cin, cout, s in self.convs:
            _, d, h, w = shapes[-1]
            assert cin == shapes[-1][0]
            shapes.append((cout, (d - 1) // s + 1, (h - 1) // s + 1, (w - 1) // s + 1))
        self.shapes = shapes
        assert self.dense[0][0] == int(np.prod(shapes[-1]))
        # flat parameter layout
        self.layout = []
        off = 0
        for n, (cin, cout, _) in enumerate(self.convs):
            for name, size in ((f"conv{n}.w", cout * cin * 27), (f"conv{n}.b", cout)):
                self.layout.append((name, off, size))
                off += size
        for n, (din, dout) in enumerate(self.dense):
            for name, size in ((f"fc{n}.w", dout * din), (f"fc{n}.b", dout)):
                self.layout.append((name, off, size))
                off += size
        self.nparams = off
        rng = np.random.default_rng(seed)
        w = np.zeros(off, np.float32)
        for name, o, size in self.layout:
            if name.endswith(".w"):
                fan_in = size // self._fan_out(name)
                w[o:o + size] = rng.normal(scale=np.sqrt(2.0 / (1 + SLOPE ** 2) / fan_in), size=size)
        self.w = torch.tensor(w, device=device)
        self.w16 = torch.zeros(off, dtype=torch.int16, device=device)
        self.g = torch.zeros(off, dtype=torch.float32, device=device)
        self.m = torch.zeros(off, dtype=torch.float32, device=device)
        self.v = torch.zeros(off, dtype=torch.float32, device=device)
        self.step = 0
        self.scratch = torch.zeros(1024, dtype=torch.float32, device=device)
        self.loss = torch.zeros(1, dtype=torch.float32, device=device)
        _ok(self.L.fwant_nn_to_bf16(_p(self.w), _p(self.w16), self.nparams, self._stream()), "to_bf16")
        self._acts = {}

    def _fan_out(self, name):
        kind, n = name.split(".")[0][:-1], int(name.split(".")[0][-1])
        if kind == "conv":
            return self.convs[n][1]
        return self.dense[n][1]

    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def view(self, t, name):
        for nm, o, size in self.layout:
            if nm == name:
                return t[o:o + size]
        raise KeyError(name)

    def params_numpy(self, bf16=True):
        """Parameters as float64 arrays shaped per layer: the values the kernels read (BF16
        weights, FP32 biases) or, with bf16=False, the FP32 master weights."""
        import torch
        w16 = (self.w16.to(torch.int32) << 16).view(torch.float32).cpu().numpy().astype(np.float64)
        w32 = self.w.cpu().numpy().astype(np.float64)
        out = {}
        for name, o, size in self.layout:
            a = (w16 if bf16 and name.endswith(".w") else w32)[o:o + size]
            if name.startswith("conv") and name.endswith(".w"):
                n = int(name[4])
                cin, cout, _ = self.convs[n]
                a = a.reshape(cout, cin, 3, 3, 3)
            elif name.startswith("fc") and name.endswith(".w"):
                din, dout = self.dense[int(name[2])]
                a = a.reshape(dout, din)
            out[name] = a
        return out

    def _buf(self, key, shape):
        t = self._acts.get(key)
        if t is None or tuple(t.shape) != tuple(shape):
            t = self.torch.zeros(shape, dtype=self.torch.float32, device=self.device)
            self._acts[key] = t
        return t

    def forward(self, x):
        """x: (B, C, D, H, W) float32 CUDA tensor -> (B, out) (kept for backward)."""
        B = x.shape[0]
        st = self._stream()
        h = x.contiguous()
        self._in = h
        outs = []
        for n, (cin, cout, s) in enumerate(self.convs):
            _, d, hh, w = self.shapes[n]
            y = self._buf(f"c{n}", (B,) + self.shapes[n + 1])
            _ok(self.L.fwant_nn_conv3d_fwd(_p(h), _p(self.view(self.w16, f"conv{n}.w")),
                                           _p(self.view(self.w, f"conv{n}.b")), _p(y), B, cin, d, hh, w, cout, s, st),
                "conv fwd")
            _ok(self.L.fwant_nn_lrelu_fwd(_p(y), y.numel(), SLOPE, st), "lrelu")
            outs.append(y)
            h = y
        h = h.reshape(B, -1)
        for n, (din, dout) in enumerate(self.dense):
            y = self._buf(f"f{n}", (B, dout))
            _ok(self.L.fwant_nn_linear_fwd(_p(h), _p(self.view(self.w16, f"fc{n}.w")),
                                           _p(self.view(self.w, f"fc{n}.b")), _p(y), B, din, dout, st), "linear fwd")
            if n + 1 < len(self.dense):
                _ok(self.L.fwant_nn_lrelu_fwd(_p(y), y.numel(), SLOPE, st), "lrelu")
            outs.append(y)
            h = y
        self._outs = outs
        if self.basis is not None:
            out = self._buf("basis_out", (B, self.G * self.T))
            _ok(self.L.fwant_nn_basis_fwd(_p(h), _p(self.basis), _p(out), B, self.G, self.K, self.T, st), "basis fwd")
            h = out
        return h

    def backward(self, dy):
        """Gradients of every parameter into self.g given d(loss)/d(output)."""
        B = dy.shape[0]
        st = self._stream()
        nc = len(self.convs)
        dy = dy.contiguous()
        if self.basis is not None:
            dc = self._buf("basis_dcoef", (B, self.G * self.K))
            _ok(self.L.fwant_nn_basis_bwd(_p(dy), _p(self.basis), _p(dc), B, self.G, self.K, self.T, st), "basis bwd")
            dy = dc
        for n in reversed(range(len(self.dense))):
            din, dout = self.dense[n]
            hin = self._outs[nc + n - 1].reshape(B, -1) if n > 0 else self._outs[nc - 1].reshape(B, -1)
            dx = self._buf(f"df{n}", (B, din))
            _ok(self.L.fwant_nn_linear_bwd(_p(hin), _p(self.view(self.w16, f"fc{n}.w")), _p(dy), _p(dx),
                                           _p(self.view(self.g, f"fc{n}.w")), _p(self.view(self.g, f"fc{n}.b")),
                                           B, din, dout, st), "linear bwd")
            _ok(self.L.fwant_nn_lrelu_bwd(_p(hin), _p(dx), dx.numel(), SLOPE, st), "lrelu bwd")
            dy = dx
        dy = dy.reshape((B,) + self.shapes[nc])
        for n in reversed(range(nc)):
            cin, cout, s = self.convs[n]
            _, d, hh, w = self.shapes[n]
            xin = self._outs[n - 1] if n > 0 else self._in
            dx = self._buf(f"dc{n}", (B,) + self.shapes[n]) if n > 0 else None
            _ok(self.L.fwant_nn_conv3d_bwd(_p(xin), _p(self.view(self.w16, f"conv{n}.w")), _p(dy), _p(dx),
                                           _p(self.view(self.g, f"conv{n}.w")), _p(self.view(self.g, f"conv{n}.b")),
                                           B, cin, d, hh, w, cout, s, st), "conv bwd")
            if n > 0:
                _ok(self.L.fwant_nn_lrelu_bwd(_p(xin), _p(dx), dx.numel(), SLOPE, st), "lrelu bwd")
                dy = dx

    def mse(self, y, t, want_grad=True):
        """(loss tensor (1,), d loss / d y or None)."""
        dy = self._buf("dy", tuple(y.shape)) if want_grad else None
        _ok(self.L.fwant_nn_mse(_p(y), _p(t), _p(dy), _p(self.loss), _p(self.scratch), y.numel(), self._stream()),
            "mse")
        return self.loss, dy

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
        self.step += 1
        _ok(self.L.fwant_nn_adam(_p(self.w), _p(self.w16), _p(self.g), _p(self.m), _p(self.v), self.nparams, lr, b1,
                                 b2, eps, wd, self.step, self._stream()), "adam")

    def train_step(self, x, t, lr, wd=0.0):
        y = self.forward(x)
        loss, dy = self.mse(y, t)
        self.backward(dy)
        self.adam(lr, wd=wd)
        return loss


def pool_volume(v, f=4, interior=3):
    """Mean over f x f x f blocks of the interior of a (nx, ny, nz) array (ghosts dropped),
    returned as (D, H, W) = (nz/f, ny/f, nx/f): depth, then the two horizontal axes."""
    a = np.asarray(v, np.float64)[interior:-interior, interior:-interior, interior:-interior]
    ni, nj, nk = (s // f * f for s in a.shape)
    a = a[:ni, :nj, :nk].reshape(ni // f, f, nj // f, f, nk // f, f).mean(axis=(1, 3, 5))
    return a.transpose(2, 1, 0).astype(np.float32)


# ---- configuration 5: data, training, screening ---------------------------------------

def c5_reference(seed=0, ni=128, nj=128, nk=64, nrecv=64, fc=0.2, t0=7.5):
    """Reference model of the surrogate workload: the layered medium without perturbation,
    a vertical surface force (Ricker fc Hz, delay t0 s) at the centre and nrecv seeded
    surface receivers sampled every 4 steps."""
    from . import inputs
    m = inputs.make_model(ni, nj, nk, seed=seed, nrecv=nrecv, perturb=0.0, fc=fc, t0=t0,
                          name=f"C5 reference {ni}x{nj}x{nk}")
    m.recv_tinv = 4
    return m


def c5_sample(ref, sample, perturb=0.05, corr_km=10.0):
    """Model `sample` of the workload: the reference with Vs scaled by 1 + dv, dv a seeded
    Gaussian-correlated field (corr_km) with max |dv| = perturb; Vp and rho unchanged.
    Returns (model, dv)."""
    from . import inputs
    rng = np.random.default_rng(1_000_003 + int(sample))
    dv = inputs.gaussian_field(ref.lam.shape, ref.x, ref.y, ref.z, corr_km, rng)
    dv *= perturb / max(np.abs(dv).max(), 1e-30)
    rho = ref.rho.astype(np.float64)
    mu0 = ref.mu.astype(np.float64)
    vp2 = (ref.lam.astype(np.float64) + 2.0 * mu0) / rho
    mu = mu0 * (1.0 + dv) ** 2
    lam = rho * vp2 - 2.0 * mu
    m = inputs.Model(**{k: getattr(ref, k) for k in ref.__dataclass_fields__})
    m.lam, m.mu = lam.astype(np.float32), mu.astype(np.float32)
    m.name = f"{ref.name} sample {sample}"
    return m, dv.astype(np.float32)


def simulate(models, nt, group=32, device=0):
    """FD solves of `models` (same grid) for nt steps, `group` at a time as one batch.
    Returns (velocity seismograms (n, 3, nsamp, nrecv) float32, device ms per solve)."""
    from . import inputs
    from ._lib import Batch, Solver
    out, ms = [], 0.0
    for g0 in range(0, len(models), group):
        sims = [inputs.attach(Solver(m.ni, m.nj, m.nk, m.stept, device=device), m) for m in models[g0:g0 + group]]
        b = Batch(sims)
        b.run(nt)
        ms += b.last_run_ms()
        for s in sims:
            out.append(s.get_seismo()[:3].copy())
        b.close()
        for s in sims:
            s.close()
    return np.stack(out), ms / len(models)


def reference_energy(ref, nt, every=8, f=4, device=0):
    """log10 of the time-integrated |v|^2 of the reference run on the pooled grid (one
    point per f^3 block), normalised to zero mean and unit deviation: (D, H, W)."""
    from . import inputs
    from ._lib import Solver
    s = inputs.attach(Solver(ref.ni, ref.nj, ref.nk, ref.stept, device=device), ref)
    subs = (inputs.LENFD + 1 + f // 2,) * 3
    subc = (ref.ni // f, ref.nj // f, ref.nk // f)
    acc = np.zeros((3,) + subc)
    done = 0
    while done < nt:
        n = min(every, nt - done)
        s.run(n)
        done += n
        v = s.get_snapshot(subs, subc, (f, f, f), comps=("Vx", "Vy", "Vz")).astype(np.float64)
        acc += v * v
    s.close()
    e = np.log10(acc.sum(axis=0) + 1e-30).transpose(2, 1, 0)
    return ((e - e.mean()) / max(e.std(), 1e-30)).astype(np.float32)


def features(dv, energy, f=4):
    """Network input of one sample: (2, D, H, W) = pooled dv x 20, reference energy."""
    return np.stack([pool_volume(dv, f) * 20.0, energy]).astype(np.float32)


def waveform_basis(u_ref, dt, fc, scale, windows=8):
    """Fixed output basis of the network: for every trace g of the reference gather
    u_ref (G, T) (sampling interval dt s), the trace and its first two time derivatives
    (scaled by 1/(2 pi fc) per derivative, i.e. to the trace's own magnitude) under
    `windows` raised-cosine windows that sum to one.  A coefficient vector then expresses
    a windowed amplitude change and time shift (to second order) of the reference wave
    trains.  Returns (G, 3 * windows, T) float32, divided by `scale`."""
    u = np.asarray(u_ref, np.float64)
    G, T = u.shape
    d1 = np.gradient(u, dt, axis=1) / (2 * np.pi * fc)
    d2 = np.gradient(d1, dt, axis=1) / (2 * np.pi * fc)
    hop = (T - 1) / (windows - 1)
    t = np.arange(T)
    win = np.zeros((windows, T))
    for w in range(windows):
        x = (t - w * hop) / hop
        win[w] = np.where(np.abs(x) < 1.0, np.cos(0.5 * np.pi * x) ** 2, 0.0)
    out = np.zeros((G, 3 * windows, T))
    for j, d in enumerate((u, d1, d2)):
        out[:, j * windows:(j + 1) * windows, :] = win[None, :, :] * d[:, None, :]
    return (out / scale).astype(np.float32)


def c5_net(in_shape, nout, seed, basis=None):
    """The surrogate network for inputs of in_shape; with a basis (G, K, T) its dense head
    emits G*K coefficients and the output is their basis expansion (nout = G*T)."""
    d, h, w = in_shape[1:]
    flat = 32 * ((((d - 1) // 2 + 1) - 1) // 2 + 1) * ((((h - 1) // 2 + 1) - 1) // 2 + 1) * \
        ((((w - 1) // 2 + 1) - 1) // 2 + 1)
    head = nout if basis is None else int(basis.shape[0] * basis.shape[1])
    return Net(in_shape, [(in_shape[0], 16, 1), (16, 32, 2), (32, 32, 2)], [(flat, 256), (256, head)], seed=seed,
               basis=basis)


class Ensemble:
    """K networks trained from different initial weights on the same data; the spread of
    their predictions estimates the error of the mean."""

    def __init__(self, in_shape, nout, k=4, seed=0, basis=None):
        self.nets = [c5_net(in_shape, nout, seed + 7919 * q, basis=basis) for q in range(k)]

    def fit(self, x, t, epochs=200, batch=32, lr=1e-3, lr_end=1e-4, wd=1e-4, seed=0):
        """x (N, C, D, H, W), t (N, out): CUDA tensors.  Returns the final epoch losses."""
        import torch
        n = x.shape[0]
        rng = np.random.default_rng(seed)
        steps = epochs * ((n + batch - 1) // batch)
        losses = []
        for q, net in enumerate(self.nets):
            it = 0
            last = 0.0
            for ep in range(epochs):
                perm = torch.tensor(rng.permutation(n), device=x.device)
                tot = torch.zeros((), device=x.device)
                for b0 in range(0, n, batch):
                    idx = perm[b0:b0 + batch]
                    a = lr + (lr_end - lr) * it / max(steps - 1, 1)
                    tot += net.train_step(x[idx], t[idx], lr=a, wd=wd)[0] * len(idx)
                    it += 1
                last = float(tot.item()) / n
            losses.append(last)
        return losses

    def predict(self, x, batch=64):
        """(mean prediction, per-sample relative spread) for x (N, ...)."""
        import torch
        preds = []
        for net in self.nets:
            outs = [net.forward(x[b0:b0 + batch]).clone() for b0 in range(0, x.shape[0], batch)]
            preds.append(torch.cat(outs))
        p = torch.stack(preds)
        mean = p.mean(dim=0)
        spread = (p - mean).pow(2).sum(dim=2).mean(dim=0).sqrt()
        return mean, spread


def generate(ref, samples, nt, energy, group=32, device=0, corr_km=10.0):
    """Inputs and FD waveforms of the given sample ids: (X (N, 2, D, H, W), U (N, 3,
    nsamp, nrecv), device ms per FD solve)."""
    xs, us, ms = [], [], []
    for g0 in range(0, len(samples), group):
        models, feats = [], []
        for n in samples[g0:g0 + group]:
            m, dv = c5_sample(ref, n, corr_km=corr_km)
            models.append(m)
            feats.append(features(dv, energy))
        u, t = simulate(models, nt, group=group, device=device)
        xs.append(np.stack(feats))
        us.append(u)
        ms.append(t * len(models))
    return np.concatenate(xs), np.concatenate(us), sum(ms) / len(samples)


def rel_err(a, b):
    """Relative L2 error of gathers a against b, per sample (first axis)."""
    a = a.reshape(a.shape[0], -1).astype(np.float64)
    b = b.reshape(b.shape[0], -1).astype(np.float64)
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


def run_c5(n_train=512, n_val=64, n_test=64, nt=800, grid=(128, 128, 64), nrecv=64, k=4, epochs=200, tol=0.01,
           seed=0, device=0, fc=0.2, t0=7.5, corr_km=25.0, windows=8, use_basis=False, log=None):
    """Train the surrogate ensemble on n_train seeded FD solves (the last n_val of them held
    back to calibrate the error estimate), then screen n_test held-out seeds: a candidate
    whose estimated error exceeds tol falls back to the FD solve.  Returns a dict of errors
    (relative L2 of the 3-component gathers), timings and the screening speedup."""
    import time

    import torch
    say = log or (lambda *a: None)
    ref = c5_reference(seed, *grid, nrecv=nrecv, fc=fc, t0=t0)
    u_ref, _ = simulate([ref], nt, device=device)
    energy = reference_energy(ref, nt, device=device)
    t0 = time.perf_counter()
    x_tr, u_tr, t_fd = generate(ref, list(range(n_train)), nt, energy, device=device, corr_km=corr_km)
    x_te, u_te, t_fd_te = generate(ref, list(range(100_000, 100_000 + n_test)), nt, energy, device=device,
                                   corr_km=corr_km)
    say(f"data: {n_train + n_test} FD solves in {time.perf_counter() - t0:.1f} s, {t_fd:.2f} ms per solve")
    # gathers trace-major: (n, 3, nrecv, nsamp), trace g = component * nrecv + receiver
    u_ref, u_tr, u_te = (np.ascontiguousarray(a.transpose(0, 1, 3, 2)) for a in (u_ref, u_tr, u_te))
    scale = float(np.sqrt(np.mean(u_ref.astype(np.float64) ** 2)))
    dev = torch.device("cuda", device)
    tgt = ((u_tr - u_ref) / scale).reshape(n_train, -1).astype(np.float32)
    X = torch.tensor(x_tr, device=dev)
    T = torch.tensor(tgt, device=dev)
    fit_n = n_train - n_val
    basis = None
    if use_basis:
        g = u_ref.reshape(-1, u_ref.shape[-1])
        basis = torch.tensor(waveform_basis(g, ref.recv_tinv * float(np.float32(ref.stept)), fc, scale, windows),
                             device=dev)
    ens = Ensemble(tuple(x_tr.shape[1:]), tgt.shape[1], k=k, seed=seed, basis=basis)
    t1 = time.perf_counter()
    losses = ens.fit(X[:fit_n], T[:fit_n], epochs=epochs, seed=seed)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    say(f"training: {k} networks x {epochs} epochs in {t_train:.1f} s, final losses {losses}")

    def gather(pred):
        return u_ref + scale * pred.cpu().numpy().reshape((-1,) + u_ref.shape[1:])

    # calibration of the error estimate on the held-back samples
    mv, sv = ens.predict(X[fit_n:])
    pv = gather(mv)
    ev = rel_err(pv, u_tr[fit_n:])
    rs = sv.cpu().numpy() * scale / np.linalg.norm(pv.reshape(len(pv), -1), axis=1)
    factor = float(np.quantile(ev / np.maximum(rs, 1e-30), 0.9))
    # screening of held-out candidates, timed on the device
    Xt = torch.tensor(x_te, device=dev)
    ens.predict(Xt)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    mt, st = ens.predict(Xt)
    e1.record()
    torch.cuda.synchronize()
    t_nn = e0.elapsed_time(e1) / n_test
    pt = gather(mt)
    err = rel_err(pt, u_te)
    base = rel_err(np.broadcast_to(u_ref, u_te.shape), u_te)
    est = factor * st.cpu().numpy() * scale / np.linalg.norm(pt.reshape(n_test, -1), axis=1)
    accept = est <= tol
    final = np.where(accept, err, 0.0)  # fallbacks are the FD solve itself
    cost = n_test * t_nn + (~accept).sum() * t_fd_te
    screening = {}
    for tq in sorted({tol, 0.01, 0.02, 0.05}):
        acc = est <= tq
        screening[f"{tq:g}"] = {
            "accepted": int(acc.sum()), "accepted_err_max": float(err[acc].max()) if acc.any() else None,
            "speedup": float(n_test * t_fd_te / (n_test * t_nn + (~acc).sum() * t_fd_te))}
    return {
        "screening": screening,
        "grid": list(grid), "nt": nt, "nrecv": nrecv, "n_train": fit_n, "n_val": n_val, "n_test": n_test,
        "corr_km": corr_km, "basis_windows": windows if use_basis else None,
        "ensemble": k, "epochs": epochs, "params_per_net": ens.nets[0].nparams,
        "fd_ms_per_solve": t_fd_te, "surrogate_ms_per_candidate": t_nn, "train_s": t_train,
        "baseline_err_median": float(np.median(base)), "baseline_err_max": float(base.max()),
        "surrogate_err_median": float(np.median(err)), "surrogate_err_max": float(err.max()),
        "surrogate_err_p90": float(np.quantile(err, 0.9)),
        "accepted": int(accept.sum()), "accepted_err_max": float(err[accept].max()) if accept.any() else None,
        "screened_err_max": float(final.max()), "error_estimate_factor": factor,
        "speedup": float(n_test * t_fd_te / cost), "tol": tol,
    }
