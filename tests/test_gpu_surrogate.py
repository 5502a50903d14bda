"""Surrogate kernels on the GPU against the FP64 restatement (oracle/surrogate_oracle.py):
forward output, loss and the gradient of every parameter, with the BF16 weights the
kernels read.  FP32 accumulation over at most a few thousand terms: 2e-5 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONVS = [(2, 4, 1), (4, 6, 2), (6, 5, 2)]
DENSE = [(5 * 3 * 2 * 2, 24), (24, 37)]
IN_SHAPE = (2, 9, 7, 5)


def _case(seed=0, B=3):
    import torch

    from fwant_gb300 import surrogate
    net = surrogate.Net(IN_SHAPE, CONVS, DENSE, seed=seed)
    # non-zero biases so that every bias gradient path is exercised
    rng = np.random.default_rng(seed + 1)
    for name, o, size in net.layout:
        if name.endswith(".b"):
            net.w[o:o + size] = torch.tensor(rng.normal(scale=0.1, size=size), dtype=torch.float32, device="cuda")
    net.L.fwant_nn_to_bf16(surrogate._p(net.w), surrogate._p(net.w16), net.nparams, net._stream())
    x = torch.tensor(rng.normal(size=(B,) + IN_SHAPE), dtype=torch.float32, device="cuda")
    t = torch.tensor(rng.normal(size=(B, DENSE[-1][1])), dtype=torch.float32, device="cuda")
    return net, x, t


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_forward_and_gradients_match_fp64(native_lib):
    import torch

    from oracle import surrogate_oracle as S
    net, x, t = _case()
    y = net.forward(x)
    loss, dy = net.mse(y, t)
    net.g.zero_()
    net.backward(dy)
    torch.cuda.synchronize()
    ref = S.Net(CONVS, DENSE, 0.1)
    p = net.params_numpy(bf16=True)
    yr, _ = ref.forward(p, x.cpu().numpy().astype(np.float64))
    assert _rel(y.cpu().numpy(), yr) < 2e-5
    lr, gr = ref.loss_and_grads(p, x.cpu().numpy().astype(np.float64), t.cpu().numpy().astype(np.float64))
    assert abs(float(loss.item()) - lr) <= 2e-5 * lr
    g = net.g.cpu().numpy()
    for name, o, size in net.layout:
        e = _rel(g[o:o + size], gr[name].reshape(-1))
        assert e < 2e-5, (name, e)


def test_training_is_deterministic_and_fits(native_lib):
    import torch
    net_a, x, t = _case(seed=4, B=8)
    net_b, _, _ = _case(seed=4, B=8)
    first = None
    for it in range(150):
        la = float(net_a.train_step(x, t, lr=3e-3).item())
        lb = float(net_b.train_step(x, t, lr=3e-3).item())
        assert la == lb
        first = la if first is None else first
    torch.cuda.synchronize()
    assert torch.equal(net_a.w, net_b.w)
    assert la < 0.05 * first, (first, la)


def test_adam_matches_formula(native_lib):
    import torch

    from fwant_gb300 import surrogate
    L = surrogate._lib()
    n = 1000
    rng = np.random.default_rng(2)
    w0 = rng.normal(size=n).astype(np.float32)
    gs = [rng.normal(size=n).astype(np.float32) for _ in range(3)]
    w = torch.tensor(w0, device="cuda")
    w16 = torch.zeros(n, dtype=torch.int16, device="cuda")
    m = torch.zeros(n, device="cuda")
    v = torch.zeros(n, device="cuda")
    lr, b1, b2, eps, wd = 1e-2, 0.9, 0.999, 1e-8, 0.01
    wr, mr, vr = w0.astype(np.float64), np.zeros(n), np.zeros(n)
    for step, gnp in enumerate(gs, start=1):
        g = torch.tensor(gnp, device="cuda")
        assert L.fwant_nn_adam(surrogate._p(w), surrogate._p(w16), surrogate._p(g), surrogate._p(m), surrogate._p(v),
                               n, lr, b1, b2, eps, wd, step, None) == 0
        mr = b1 * mr + (1 - b1) * gnp
        vr = b2 * vr + (1 - b2) * gnp.astype(np.float64) ** 2
        wr = wr * (1 - lr * wd) - lr * (mr / (1 - b1 ** step)) / (np.sqrt(vr / (1 - b2 ** step)) + eps)
    torch.cuda.synchronize()
    np.testing.assert_allclose(w.cpu().numpy(), wr, rtol=1e-5, atol=1e-6)
    from oracle import surrogate_oracle as S
    bits = (w16.to(torch.int32) << 16).view(torch.float32).cpu().numpy()
    np.testing.assert_array_equal(bits, S.bf16_round(w.cpu().numpy()).astype(np.float32))


def test_surrogate_beats_reference_waveforms(native_lib):
    """What the trained network gains: on held-out perturbed models its waveforms are
    closer to the FD solve than the reference-model waveforms (the screening answer
    without the network).  Small configuration of the 128x128x64 workload."""
    from fwant_gb300 import surrogate
    r = surrogate.run_c5(n_train=96, n_val=16, n_test=16, nt=240, grid=(40, 40, 24), nrecv=12, k=2, epochs=60,
                         fc=0.5, t0=2.5, use_basis=True)
    print(r)
    assert r["baseline_err_median"] > 0.005  # the perturbations change the waveforms
    assert r["surrogate_err_median"] < 0.7 * r["baseline_err_median"]


def test_basis_layer_matches_numpy(native_lib):
    import torch

    from fwant_gb300 import surrogate
    rng = np.random.default_rng(9)
    B, G, K, T = 3, 5, 7, 11
    coef = rng.normal(size=(B, G, K)).astype(np.float32)
    basis = rng.normal(size=(G, K, T)).astype(np.float32)
    dout = rng.normal(size=(B, G, T)).astype(np.float32)
    c, bs, d = (torch.tensor(a, device="cuda") for a in (coef, basis, dout))
    out = torch.zeros((B, G, T), device="cuda")
    dc = torch.zeros((B, G, K), device="cuda")
    L = surrogate._lib()
    assert L.fwant_nn_basis_fwd(surrogate._p(c), surrogate._p(bs), surrogate._p(out), B, G, K, T, None) == 0
    assert L.fwant_nn_basis_bwd(surrogate._p(d), surrogate._p(bs), surrogate._p(dc), B, G, K, T, None) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(out.cpu().numpy(), np.einsum("bgk,gkt->bgt", coef, basis), rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(dc.cpu().numpy(), np.einsum("bgt,gkt->bgk", dout, basis), rtol=1e-5, atol=1e-5)
