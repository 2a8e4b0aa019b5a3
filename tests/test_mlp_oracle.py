"""The MLP oracle's backward pass against central finite differences (FP64,
no rounding) — checks the gradient formulas the GPU kernels implement."""
import numpy as np

from oracle import mlp_oracle as mo


def tiny_layers(rng, dims):
    return [(rng.standard_normal((dims[i + 1], dims[i])) * 0.5, rng.standard_normal(dims[i + 1]) * 0.1)
            for i in range(len(dims) - 1)]


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    dims = [4, 8, 8, 3]
    layers = tiny_layers(rng, dims)
    X = rng.standard_normal((16, 4))
    T = rng.standard_normal((16, 3))
    _, _, grads = mo.forward_backward(layers, X, T, n_out=3, exact=True)
    h = 1e-6
    for l, (W, b) in enumerate(layers):
        for arr, g in ((W, grads[l][0]), (b, grads[l][1])):
            idx = [tuple(rng.integers(0, s) for s in arr.shape) for _ in range(5)]
            for ix in idx:
                old = arr[ix]
                arr[ix] = old + h
                lp = mo.forward_backward(layers, X, T, 3, exact=True)[1]
                arr[ix] = old - h
                lm = mo.forward_backward(layers, X, T, 3, exact=True)[1]
                arr[ix] = old
                fd = (lp - lm) / (2 * h)
                assert abs(fd - g[ix]) <= 1e-6 * max(1.0, abs(fd)), (l, ix, fd, g[ix])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e38], np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == -2.5
