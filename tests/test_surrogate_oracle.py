"""The FP64 restatement of the surrogate network: its hand-derived backward against
central finite differences, its convolution against a direct loop, and the BF16 rounding
against known bit patterns."""
import numpy as np


def _net():
    from oracle import surrogate_oracle as S
    return S, S.Net(convs=[(2, 3, 1), (3, 4, 2)], dense=[(4 * 3 * 3 * 2, 7), (7, 5)], slope=0.1)


def _params(rng, net):
    p = {}
    for n, (ci, co, _) in enumerate(net.convs):
        p[f"conv{n}.w"] = rng.normal(scale=0.4, size=(co, ci, 3, 3, 3))
        p[f"conv{n}.b"] = rng.normal(scale=0.1, size=co)
    for n, (di, do) in enumerate(net.dense):
        p[f"fc{n}.w"] = rng.normal(scale=0.4, size=(do, di))
        p[f"fc{n}.b"] = rng.normal(scale=0.1, size=do)
    return p


def test_backward_matches_finite_differences():
    S, net = _net()
    rng = np.random.default_rng(0)
    p = _params(rng, net)
    x = rng.normal(size=(2, 2, 6, 5, 4))
    t = rng.normal(size=(2, 5))
    _, g = net.loss_and_grads(p, x, t)
    h = 1e-6
    for name, a in p.items():
        flat = a.reshape(-1)
        for idx in rng.choice(flat.size, size=min(6, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + h
            lp, _ = net.loss_and_grads(p, x, t)
            flat[idx] = old - h
            lm, _ = net.loss_and_grads(p, x, t)
            flat[idx] = old
            fd = (lp - lm) / (2 * h)
            an = g[name].reshape(-1)[idx]
            assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)), (name, idx, fd, an)


def test_conv_against_direct_loop():
    S, _ = _net()
    rng = np.random.default_rng(1)
    x = rng.normal(size=(1, 2, 5, 4, 3))
    w = rng.normal(size=(3, 2, 3, 3, 3))
    b = rng.normal(size=3)
    for s in (1, 2):
        y = S.conv3d(x, w, b, s)
        for o in range(3):
            for d in range(y.shape[2]):
                for hh in range(y.shape[3]):
                    for ww in range(y.shape[4]):
                        acc = b[o]
                        for c in range(2):
                            for kd in range(3):
                                for kh in range(3):
                                    for kw in range(3):
                                        di, hi, wi = d * s + kd - 1, hh * s + kh - 1, ww * s + kw - 1
                                        if 0 <= di < 5 and 0 <= hi < 4 and 0 <= wi < 3:
                                            acc += w[o, c, kd, kh, kw] * x[0, c, di, hi, wi]
                        assert abs(y[0, o, d, hh, ww] - acc) < 1e-12


def test_bf16_rounding():
    S, _ = _net()
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e38, 1e-40], np.float32)
    got = S.bf16_round(vals)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: to even (1); 1 + 3*2^-9 rounds up
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 ** -7 and got[3] == -2.5
    assert abs(got[4] - 3.0e38) / 3.0e38 < 2 ** -8
