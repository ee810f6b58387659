"""The FP64 oracle of the warm-start network: its hand-written backward pass
against central differences (the oracle is what the GPU gradients are checked
against in test_gpu_surrogate.py)."""
import numpy as np

from oracle import cnn_oracle as co


def tiny_params(rng, widths=(3, 4, 4, 5, 5), cin=2, cout=3):
    w = widths
    shapes = [(w[0], cin), (w[0], w[0])] + [(w[i], w[i - 1]) for i in range(1, 5)] + \
             [(w[i], w[i + 1]) for i in range(3, -1, -1)] + [(cout, w[0])]
    return [(rng.standard_normal((o, i, 3, 3)) * 0.4, rng.standard_normal(o) * 0.1) for o, i in shapes]


def test_oracle_backward_matches_central_differences():
    rng = np.random.default_rng(5)
    params = tiny_params(rng)
    x = rng.standard_normal((2, 2, 16, 16))
    t = rng.standard_normal((2, 3, 16, 16))
    mask = (rng.random((2, 16, 16)) > 0.3).astype(float)

    def loss_of(ps):
        net = co.Net(ps)
        return co.masked_loss(net.forward(x), t, mask)[0]

    net = co.Net(params)
    _, dp = co.masked_loss(net.forward(x), t, mask)
    grads = net.backward(dp)

    def central(layer, which, idx):
        # a ReLU kink can sit inside a wide stencil: the closest of several widths counts
        best = np.inf
        for eps in (1e-5, 1e-7, 1e-9):
            pp = [[ww.copy(), bb.copy()] for ww, bb in params]
            pm = [[ww.copy(), bb.copy()] for ww, bb in params]
            pp[layer][which][idx] += eps
            pm[layer][which][idx] -= eps
            num = (loss_of(pp) - loss_of(pm)) / (2 * eps)
            best = min(best, abs(num - grads[layer][which][idx]) / max(1.0, abs(num)))
        return best

    for layer in range(len(params)):
        w, b = params[layer]
        for idx in [(0, 0, 1, 1), (w.shape[0] - 1, w.shape[1] - 1, 2, 0)]:
            assert central(layer, 0, idx) <= 1e-5
        assert central(layer, 1, (0,)) <= 1e-5
