"""FP64 NumPy restatement of the warm-start network -- TEST INFRASTRUCTURE
ONLY (gradient checks of libmantiis_cnn.so in tests/); never used by the
product.

It follows mantiis_gb300/surrogate.py layer by layer: 3x3 convolutions with
zero padding (weights [Cout][Cin][3][3], offsets (kx - 1, ky - 1) for
k = 3 ky + kx), ReLU, 2x2 mean pooling, nearest 2x upsampling, skip
connections by addition, and the masked mean squared error.  The network has
no counterpart in the reference; the oracle's backward pass is pinned by
central differences in its own test.
"""
import numpy as np


def conv3x3(x, w, b):
    """x: (n, cin, h, wd), w: (cout, cin, 3, 3), b: (cout,) -> (n, cout, h, wd)."""
    n, cin, h, wd = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    y = np.zeros((n, w.shape[0], h, wd))
    for ky in range(3):
        for kx in range(3):
            y += np.einsum("oc,nchw->nohw", w[:, :, ky, kx], xp[:, :, ky:ky + h, kx:kx + wd])
    return y + b[None, :, None, None]


def conv3x3_backward(x, w, dy):
    """Gradients of conv3x3 with respect to x, w and b."""
    n, cin, h, wd = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    dxp = np.zeros_like(xp)
    dw = np.zeros_like(w)
    for ky in range(3):
        for kx in range(3):
            dw[:, :, ky, kx] = np.einsum("nohw,nchw->oc", dy, xp[:, :, ky:ky + h, kx:kx + wd])
            dxp[:, :, ky:ky + h, kx:kx + wd] += np.einsum("oc,nohw->nchw", w[:, :, ky, kx], dy)
    return dxp[:, :, 1:-1, 1:-1], dw, dy.sum(axis=(0, 2, 3))


def pool(x):
    n, c, h, wd = x.shape
    return x.reshape(n, c, h // 2, 2, wd // 2, 2).mean(axis=(3, 5))


def pool_backward(dy):
    return np.repeat(np.repeat(dy, 2, axis=2), 2, axis=3) * 0.25


def up(x):
    return np.repeat(np.repeat(x, 2, axis=2), 2, axis=3)


def up_backward(dy):
    n, c, h, wd = dy.shape
    return dy.reshape(n, c, h // 2, 2, wd // 2, 2).sum(axis=(3, 5))


def relu(x):
    return np.maximum(x, 0.0)


class Net:
    """The same layers as surrogate.UNet; params: list of (w, b) in its layer order
    (enc0a, enc0b, enc[1..4], dec[levels 3..0], out)."""

    def __init__(self, params):
        self.params = [(np.asarray(w, np.float64), np.asarray(b, np.float64)) for w, b in params]

    def forward(self, x):
        P = self.params
        a = {"x": x}
        a["a0"] = relu(conv3x3(x, *P[0]))
        e = [relu(conv3x3(a["a0"], *P[1]))]
        p = [None]
        for i in range(1, 5):
            p.append(pool(e[i - 1]))
            e.append(relu(conv3x3(p[i], *P[1 + i])))
        d = {4: e[4]}
        u, c = {}, {}
        for k, i in enumerate(range(3, -1, -1)):
            u[i] = up(d[i + 1])
            c[i] = relu(conv3x3(u[i], *P[6 + k]))
            d[i] = c[i] + e[i]
        y = conv3x3(d[0], *P[10])
        a.update(e=e, p=p, u=u, c=c, d=d)
        self.a = a
        return y

    def backward(self, dy):
        """Weight and bias gradients, in layer order."""
        P, a = self.params, self.a
        e, p, u, c, d = a["e"], a["p"], a["u"], a["c"], a["d"]
        grads = [None] * len(P)
        dd, gw, gb = conv3x3_backward(d[0], P[10][0], dy)
        grads[10] = (gw, gb)
        de = {}
        for i in range(0, 4):
            de[i] = dd.copy()
            dc = dd * (c[i] > 0)
            k = 3 - i
            du, gw, gb = conv3x3_backward(u[i], P[6 + k][0], dc)
            grads[6 + k] = (gw, gb)
            dd = up_backward(du)
        de[4] = dd
        for i in range(4, 0, -1):
            g = de[i] * (e[i] > 0)
            dp, gw, gb = conv3x3_backward(p[i], P[1 + i][0], g)
            grads[1 + i] = (gw, gb)
            de[i - 1] = de[i - 1] + pool_backward(dp)
        g = de[0] * (e[0] > 0)
        da0, gw, gb = conv3x3_backward(a["a0"], P[1][0], g)
        grads[1] = (gw, gb)
        g = da0 * (a["a0"] > 0)
        _, gw, gb = conv3x3_backward(a["x"], P[0][0], g)
        grads[0] = (gw, gb)
        return grads


def masked_loss(pred, target, mask):
    """Mean over fluid pixels and channels of the squared error, and its gradient."""
    n, ch = pred.shape[:2]
    norm = max(float(mask.sum()) * ch, 1.0)
    d = (pred - target) * mask[:, None]
    return float((d * d).sum() / norm), 2.0 * d / norm
