"""Learned warm start for the steady transport state.

An encoder-decoder CNN (4 pooling levels down, 4 upsampling levels up, widths
32-64-128-256 with a 256-wide bottleneck, skip connections by addition) maps a
pore image and its log Knudsen-number map to the steady velocity and density
fields.  Its forward and backward passes run on the kernels of
libmantiis_cnn.so (include/mantiis_cnn.h): 3x3 convolutions with BF16 weights
and FP32 accumulation, pooling, upsampling, ReLU, a masked squared-error loss
and Adam.  PyTorch only holds the device buffers.

The prediction only initialises the lattice Boltzmann state (f = f_eq of the
predicted fields, with the mass of the solver's own start); the solver then
iterates to its own convergence criterion, so every reported field and
permeability is the solver's converged result.  The reference has no
counterpart: it always starts from rest (include/coreLB.hpp:381-417).

Targets are scaled so that they do not depend on the body force or the mean
viscosity: u * nu_mean / F_body and (rho - rho_in) * nu_mean / F_body.  Pore
velocities are heavy-tailed (throats carry orders of magnitude more than dead
ends), so the network learns asinh(target / scale) with a per-channel scale
(UNet.scale, the median magnitude of the training targets).
"""
import ctypes as C
import os
import time
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libmantiis_cnn.so"
_cnn = None
# True: the convolutions' forward and data gradient run as the tcgen05 implicit
# GEMMs (cnn_conv3x3_*_tc).  Their operand staging (the threads gather the patch
# matrix and split it into two BF16 parts in shared memory, one stage) bounds
# them at 6-12 TFLOP/s, below the CUDA-core kernels' 10-14.5 at this network's
# layer sizes (8 x 32..256 channels, 16^2..128^2 pixels; bench.py --conv), so
# those stay the default; both agree with FP64 to within 6e-6 of the largest
# output.
TENSOR_CORES = False

_P = C.c_void_p
_SIG = {
    "cnn_conv3x3_forward": [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P],
    "cnn_conv3x3_backward_data": [_P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P],
    "cnn_conv3x3_forward_tc": [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P],
    "cnn_conv3x3_backward_data_tc": [_P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P],
    "cnn_conv3x3_backward_weight_tc": [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P],
    "cnn_tc_error": [],
    "cnn_conv3x3_backward_weight": [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P],
    "cnn_relu_backward": [_P, _P, C.c_int64, _P],
    "cnn_avgpool2_forward": [_P, _P, C.c_int, C.c_int, C.c_int, _P],
    "cnn_avgpool2_backward": [_P, _P, C.c_int, C.c_int, C.c_int, _P],
    "cnn_upsample2_forward": [_P, _P, C.c_int, C.c_int, C.c_int, _P],
    "cnn_upsample2_backward": [_P, _P, C.c_int, C.c_int, C.c_int, _P],
    "cnn_add": [_P, _P, C.c_int64, _P],
    "cnn_mse": [_P, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, _P],
    "cnn_adam": [_P, _P, _P, _P, _P, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, _P],
    "cnn_to_bf16": [_P, _P, C.c_int64, _P],
}


def cnn_lib():
    """Loads libmantiis_cnn.so (raises if it has not been built)."""
    global _cnn
    if _cnn is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with mantiis_gb300.build.build() first")
        L = C.CDLL(str(LIB_PATH))
        for name, args in _SIG.items():
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = args
        _cnn = L
    return _cnn


def _ptr(t):
    """Device address of a contiguous CUDA tensor (the kernels take FP32 data or BF16 bits)."""
    if t is None:
        return None
    import torch

    if not (t.is_cuda and t.is_contiguous() and t.dtype in (torch.float32, torch.int16)):
        raise TypeError(f"expected a contiguous float32 / int16 CUDA tensor, got {t.dtype} {tuple(t.shape)}")
    return C.c_void_p(t.data_ptr())


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with status {rc}")


def _stream():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class Conv3x3:
    """3x3 convolution: FP32 master weights (for Adam), BF16 copy (for the kernels)."""

    def __init__(self, cin, cout, rng, scale=None):
        import torch

        self.cin, self.cout = cin, cout
        std = scale if scale is not None else np.sqrt(2.0 / (9 * cin))
        w = (rng.standard_normal((cout, cin, 3, 3)) * std).astype(np.float32)
        self.w = torch.tensor(w, dtype=torch.float32, device="cuda")
        self.b = torch.zeros(cout, dtype=torch.float32, device="cuda")
        self.w16 = torch.empty(w.size, dtype=torch.int16, device="cuda")
        self.dw = torch.zeros_like(self.w)
        self.db = torch.zeros_like(self.b)
        self.state = [torch.zeros_like(self.w), torch.zeros_like(self.w), torch.zeros_like(self.b),
                      torch.zeros_like(self.b)]
        self.sync_bf16()

    def sync_bf16(self):
        _check(cnn_lib().cnn_to_bf16(_ptr(self.w), _ptr(self.w16), self.w.numel(), _stream()), "to_bf16")

    def forward(self, x, relu):
        import torch

        n, _, h, w = x.shape
        y = torch.empty((n, self.cout, h, w), dtype=torch.float32, device="cuda")
        fwd = cnn_lib().cnn_conv3x3_forward_tc if TENSOR_CORES else cnn_lib().cnn_conv3x3_forward
        _check(fwd(_ptr(x), _ptr(self.w16), _ptr(self.b), _ptr(y), n, self.cin, self.cout, h, w, 1 if relu else 0,
                   _stream()), "conv forward")
        return y

    def backward(self, x, dy, need_dx=True):
        """Accumulates dw, db from the layer input x and output gradient dy; returns dx."""
        import torch

        n, _, h, w = x.shape
        L = cnn_lib()
        _check(L.cnn_conv3x3_backward_weight(_ptr(x), _ptr(dy), _ptr(self.dw), _ptr(self.db), n, self.cin, self.cout,
                                             h, w, _stream()), "conv weight gradient")
        if not need_dx:
            return None
        dx = torch.empty_like(x)
        bwd = L.cnn_conv3x3_backward_data_tc if TENSOR_CORES else L.cnn_conv3x3_backward_data
        _check(bwd(_ptr(dy), _ptr(self.w16), _ptr(dx), n, self.cin, self.cout, h, w, _stream()), "conv data gradient")
        return dx

    def zero_grad(self):
        self.dw.zero_()
        self.db.zero_()

    def adam(self, lr, step, b1=0.9, b2=0.999, eps=1e-8):
        L = cnn_lib()
        _check(L.cnn_adam(_ptr(self.w), _ptr(self.dw), _ptr(self.state[0]), _ptr(self.state[1]), _ptr(self.w16),
                          self.w.numel(), lr, b1, b2, eps, step, _stream()), "adam")
        _check(L.cnn_adam(_ptr(self.b), _ptr(self.db), _ptr(self.state[2]), _ptr(self.state[3]), None,
                          self.b.numel(), lr, b1, b2, eps, step, _stream()), "adam")


def _relu_bw(dy, y):
    _check(cnn_lib().cnn_relu_backward(_ptr(dy), _ptr(y), dy.numel(), _stream()), "relu backward")
    return dy


def _pool(x):
    import torch

    n, c, h, w = x.shape
    y = torch.empty((n, c, h // 2, w // 2), dtype=torch.float32, device="cuda")
    _check(cnn_lib().cnn_avgpool2_forward(_ptr(x), _ptr(y), n * c, h, w, _stream()), "pool")
    return y


def _pool_bw(dy, shape):
    import torch

    n, c, h, w = shape
    dx = torch.empty(shape, dtype=torch.float32, device="cuda")
    _check(cnn_lib().cnn_avgpool2_backward(_ptr(dy), _ptr(dx), n * c, h, w, _stream()), "pool backward")
    return dx


def _up(x):
    import torch

    n, c, h, w = x.shape
    y = torch.empty((n, c, 2 * h, 2 * w), dtype=torch.float32, device="cuda")
    _check(cnn_lib().cnn_upsample2_forward(_ptr(x), _ptr(y), n * c, h, w, _stream()), "upsample")
    return y


def _up_bw(dy):
    import torch

    n, c, h2, w2 = dy.shape
    dx = torch.empty((n, c, h2 // 2, w2 // 2), dtype=torch.float32, device="cuda")
    _check(cnn_lib().cnn_upsample2_backward(_ptr(dy), _ptr(dx), n * c, h2 // 2, w2 // 2, _stream()),
           "upsample backward")
    return dx


def _add(y, x):
    _check(cnn_lib().cnn_add(_ptr(y), _ptr(x), y.numel(), _stream()), "add")
    return y


class UNet:
    """Encoder-decoder of widths w0..w3 and bottleneck w4; input 2 channels
    (pore, scaled log Kn), output 3 channels (scaled u_x, u_y, rho - rho_in).
    Image sides must be multiples of 16."""

    def __init__(self, widths=(32, 64, 128, 256, 256), cin=2, cout=3, seed=0):
        rng = np.random.default_rng(seed)
        w = widths
        self.widths = tuple(widths)
        self.enc0a = Conv3x3(cin, w[0], rng)
        self.enc0b = Conv3x3(w[0], w[0], rng)
        self.enc = [Conv3x3(w[i - 1], w[i], rng) for i in range(1, 5)]  # after pooling, levels 1..4
        self.dec = [Conv3x3(w[i + 1], w[i], rng) for i in range(3, -1, -1)]  # after upsampling, levels 3..0
        self.out = Conv3x3(w[0], cout, rng, scale=np.sqrt(1.0 / (9 * w[0])))
        self.step = 0
        self.scale = np.ones(3)  # target scaling (set from the training data)

    def layers(self):
        return [self.enc0a, self.enc0b, *self.enc, *self.dec, self.out]

    def forward(self, x, keep=False):
        a = {"x": x}
        a["a0"] = self.enc0a.forward(x, True)
        e = [self.enc0b.forward(a["a0"], True)]
        p = [None]
        for i in range(1, 5):
            p.append(_pool(e[i - 1]))
            e.append(self.enc[i - 1].forward(p[i], True))
        d = {4: e[4]}
        u, c = {}, {}
        for k, i in enumerate(range(3, -1, -1)):
            u[i] = _up(d[i + 1])
            c[i] = self.dec[k].forward(u[i], True)
            d[i] = _add(c[i].clone(), e[i])
        y = self.out.forward(d[0], False)
        if keep:
            a.update(e=e, p=p, u=u, c=c, d=d)
            self._acts = a
        return y

    def backward(self, dy):
        a = self._acts
        e, p, u, c, d = a["e"], a["p"], a["u"], a["c"], a["d"]
        dd = self.out.backward(d[0], dy)
        de = {}
        for i in range(0, 4):
            # d[i] = c[i] + e[i]: the gradient reaches the skip and the decoder conv
            de[i] = dd.clone()
            dc = _relu_bw(dd, c[i])
            du = self.dec[3 - i].backward(u[i], dc)
            dd = _up_bw(du)  # gradient of d[i + 1]
        de[4] = dd
        for i in range(4, 0, -1):
            g = _relu_bw(de[i], e[i])
            dp = self.enc[i - 1].backward(p[i], g)
            _add(de[i - 1], _pool_bw(dp, tuple(e[i - 1].shape)))
        g = _relu_bw(de[0], e[0])
        da0 = self.enc0b.backward(a["a0"], g)
        g = _relu_bw(da0, a["a0"])
        self.enc0a.backward(a["x"], g, need_dx=False)

    def zero_grad(self):
        for l in self.layers():
            l.zero_grad()

    def adam(self, lr):
        self.step += 1
        for l in self.layers():
            l.adam(lr, self.step)


def masked_loss(pred, target, mask):
    """Mean squared error over fluid pixels and channels; returns (loss, dpred)."""
    import torch

    n, ch, h, w = pred.shape
    norm = float(mask.sum().item()) * ch
    dp = torch.empty_like(pred)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    _check(cnn_lib().cnn_mse(_ptr(pred), _ptr(target), _ptr(mask), _ptr(dp), _ptr(loss), n, ch, h, w,
                             max(norm, 1.0), _stream()), "loss")
    return loss, dp


# ---- data: scaled inputs and targets, the solver's steady fields


def network_input(pore, kn):
    """2 x n x n: the void mask and log10(Kn) / 2 on void pixels."""
    void = (pore == 1).astype(np.float32)
    lk = np.where(pore == 1, np.log10(np.maximum(kn, 1e-12)) / 2.0, 0.0).astype(np.float32)
    return np.stack([void, lk])


def field_scale(solver):
    """nu_mean / F_body of a solver: u * scale does not depend on the forcing."""
    nu = (solver.info["tau_mean"] - 0.5) / 3.0
    return nu / solver.params.fbody


def steady_targets(solver):
    """3 x n x n targets from a solver's current fields (before the dataset constant)."""
    px = solver.pixels()
    s = field_scale(solver)
    void = px["rho"] != 0
    drho = np.where(void, px["rho"] - solver.info["rho_in"], 0.0)
    return np.stack([px["ux"] * s, px["uy"] * s, drho * s]).astype(np.float32)


def run_to_steady(solver, chunk=1000, tol=1e-6, max_steps=200000):
    """Advances in chunks until the permeability changes by less than tol
    (relative) over one chunk.  Returns (steps, seconds spent stepping, the
    host waiting for each chunk, permeability)."""
    steps, secs = 0, 0.0
    k_old = solver.observables()["permeability"]
    while steps < max_steps:
        t0 = time.perf_counter()
        solver.advance_graph(chunk)
        solver.sync()
        secs += time.perf_counter() - t0
        steps += chunk
        k = solver.observables()["permeability"]
        if k != 0 and abs(k - k_old) <= tol * abs(k):
            return steps, secs, k
        k_old = k
    return steps, secs, k_old


def run_batch_to_steady(batch, chunk=1000, tol=1e-6, max_steps=200000, drop_settled=True, stats=None):
    """run_to_steady for a batch: the images advance together, `chunk` steps at a
    time, until each one's permeability has settled (relative change <= tol over
    a chunk).  With drop_settled an image leaves the batch when it settles (the
    rest continue in a batch of their own, on the same stream and engine), so its
    state is the one at which it settled and it costs no further GPU time; else
    settled images keep stepping with the rest.  Returns per image the step
    count at which it settled (max_steps if never) and the permeabilities; `stats`
    (a dict) receives the lattice updates done ("lu") and the batches built."""
    from .native import Batch

    solvers = list(batch.solvers)
    n = len(solvers)
    lu_of = np.array([float(s.info["lu_per_step"]) for s in solvers])
    k_old = np.array([o["permeability"] for o in batch.observables()])
    k_now = k_old.copy()
    done = np.zeros(n, bool)
    steps_at = np.full(n, max_steps)
    active = np.arange(n)
    cur, own = batch, False
    lu, batches = 0.0, 1
    steps = 0
    try:
        while steps < max_steps and not done.all():
            cur.advance(chunk)
            cur.sync()
            steps += chunk
            lu += chunk * lu_of[active].sum()
            k = np.array([o["permeability"] for o in cur.observables()])
            newly = (~done[active]) & np.isfinite(k) & (k != 0) & (np.abs(k - k_old[active]) <= tol * np.abs(k))
            steps_at[active[newly]] = steps
            done[active[newly]] = True
            k_now[active] = k
            k_old[active] = k
            if drop_settled and newly.any() and not done.all():
                active = active[~newly]
                nxt = Batch([solvers[i] for i in active])
                if batch.stream is not None:
                    nxt.set_stream(batch.stream)
                if batch.engine is not None:
                    nxt.set_engine(*batch.engine)
                if own:
                    cur.close()
                cur, own = nxt, True
                batches += 1
    finally:
        if own:
            cur.close()
    if stats is not None:
        stats.update(lu=lu, batches=batches)
    return steps_at, k_now


def target_scale(targets, masks):
    """Per-channel scale of the encoding: median |target| over fluid pixels."""
    return np.array([np.median(np.abs(targets[:, c][masks > 0])) + 1e-30 for c in range(targets.shape[1])])


def encode(targets, scale):
    return np.arcsinh(targets / scale[None, :, None, None]).astype(np.float32)


def predict(net, pore, kn):
    """Network prediction (3 x n x n, in target units)."""
    import torch

    x = torch.tensor(network_input(pore, kn)[None], dtype=torch.float32, device="cuda")
    y = net.forward(x).cpu().numpy()[0].astype(np.float64)
    return np.sinh(y) * net.scale[:, None, None]


def warm_start(solver, net, pore, kn, use_density=False):
    """Sets the solver's state to f_eq of the predicted velocity at each cell's
    top-left pixel, with the solver's own initial density rho_in.  The steady
    density deviations are tiny, and an inexact predicted density field only
    adds a slow pressure relaxation; use_density=True takes it anyway, shifted
    to the mass of the solver's own start (a closed x-periodic system settles to
    the steady state of its mass)."""
    y = predict(net, pore, kn)
    s = field_scale(solver)
    cx, cy, lv = solver.cell_positions()
    ux = y[0][cy, cx] / s
    uy = y[1][cy, cx] / s
    rho = np.full(ux.shape, solver.info["rho_in"])
    if use_density:
        drho = y[2][cy, cx] / s
        area = 4.0 ** (lv - 1)
        rho = rho + drho - (drho * area).sum() / area.sum()
    solver.set_equilibrium(rho, ux, uy)


def train(net, inputs, targets, masks, epochs=20, batch=8, lr=1e-3, seed=0, log=None):
    """Adam on the masked squared error; inputs / targets / masks are arrays
    (N x 2 x n x n, N x 3 x n x n, N x n x n) of scaled data.  Returns the
    mean loss of each epoch."""
    import torch

    rng = np.random.default_rng(seed)
    X = torch.tensor(np.asarray(inputs, np.float32), device="cuda")
    Y = torch.tensor(np.asarray(targets, np.float32), device="cuda")
    M = torch.tensor(np.asarray(masks, np.float32), device="cuda")
    history = []
    t0 = time.perf_counter()
    for ep in range(epochs):
        order = rng.permutation(len(X))
        tot = 0.0
        for b0 in range(0, len(order), batch):
            idx = torch.tensor(order[b0:b0 + batch], device="cuda")
            x, y, m = X[idx].contiguous(), Y[idx].contiguous(), M[idx].contiguous()
            net.zero_grad()
            p = net.forward(x, keep=True)
            loss, dp = masked_loss(p, y, m)
            net.backward(dp)
            net.adam(lr)
            tot += float(loss.item()) * len(idx)
        history.append(tot / len(order))
        if log:
            log(f"epoch {ep + 1}: loss {history[-1]:.4e} ({time.perf_counter() - t0:.1f} s)")
    return history


# ---- end-to-end: data from the batched solver, training, warm vs cold


def synthetic_image(n, seed, porosity, kn_mean):
    """Seeded disk image (void x-edge columns, see MGPU_DISKS_OPEN_X_EDGES) with
    its local pore size, Kn map and the dx that gives the drawn mean Kn."""
    from .native import generate_disks, pore_properties, units

    pore = generate_disks(n, max(2, n // 64), max(4, n // 16), porosity, seed, open_x_edges=True)
    H, ku = pore_properties(pore, 1.0, 1.0)
    void = pore == 1
    mfp = units()["mfp"]
    dx = mfp * ku[void].mean() / kn_mean
    return dict(pore=pore, kn=np.where(void, ku * mfp / dx, 0.0), locpore=H, dx=float(dx))


def make_dataset(n, count, seed0=1000, chunk=500, tol=1e-6, max_steps=100000, log=None):
    """Steady single-block fields of `count` seeded n x n images (porosity
    U[0.5, 0.7], mean Kn log-uniform in [0.05, 1]), all stepped as one batch.
    Images that do not settle are left out.  Returns X, Y (unencoded), M."""
    from .native import Batch, Solver, default_params

    rng = np.random.default_rng(seed0)
    imgs = [synthetic_image(n, seed0 + i, rng.uniform(0.5, 0.7), float(np.exp(rng.uniform(np.log(0.05), 0.0))))
            for i in range(count)]
    sol = [Solver(d["pore"], d["kn"], d["locpore"], default_params(dx=d["dx"])) for d in imgs]
    b = Batch(sol)
    t0 = time.perf_counter()
    steps, _ = run_batch_to_steady(b, chunk=chunk, tol=tol, max_steps=max_steps)
    X = np.stack([network_input(d["pore"], d["kn"]) for d in imgs])
    Y = np.stack([steady_targets(s) for s in sol])
    M = np.stack([(d["pore"] == 1) for d in imgs]).astype(np.float32)
    good = np.isfinite(Y).all(axis=(1, 2, 3)) & (steps < max_steps)
    if log:
        log(f"data: {count} images {n}^2 settled in {int(steps[good].max()) if good.any() else 0} steps "
            f"({time.perf_counter() - t0:.1f} s), kept {int(good.sum())}")
    b.close()
    for s in sol:
        s.close()
    return X[good], Y[good], M[good]


def evaluate(net, n, count, seed0=90000, chunk=500, tol=1e-6, max_steps=200000, log=None):
    """Cold start (rest) against warm start (network prediction) on held-out
    images: steps and seconds to the permeability criterion, and the relative
    difference of the two converged permeabilities."""
    from .native import Solver, default_params

    out = []
    for i in range(count):
        d = synthetic_image(n, seed0 + i, 0.6, 0.05 + 0.95 * i / max(1, count - 1))
        p = default_params(dx=d["dx"])
        cold = Solver(d["pore"], d["kn"], d["locpore"], p)
        sc, tc, kc = run_to_steady(cold, chunk, tol, max_steps)
        warm = Solver(d["pore"], d["kn"], d["locpore"], p)
        t0 = time.perf_counter()
        warm_start(warm, net, d["pore"], d["kn"])
        t_pred = time.perf_counter() - t0
        sw, tw, kw = run_to_steady(warm, chunk, tol, max_steps)
        tgt = steady_targets(cold)
        pred = predict(net, d["pore"], d["kn"])
        void = d["pore"] == 1
        err = float(np.abs(pred[0] - tgt[0])[void].mean() / max(np.abs(tgt[0])[void].mean(), 1e-30))
        out.append(dict(cold_steps=int(sc), warm_steps=int(sw), cold_s=tc, warm_s=tw + t_pred,
                        permeability_rel_diff=abs(kw - kc) / abs(kc), prediction_rel_err=err))
        if log:
            log(str(out[-1]))
        cold.close()
        warm.close()
    return out


# ---- config 5: the network trained on the config-4 set's steady fields and
# used on held-out 1024^2 multi-block images


def solver_params(d, **kw):
    """Parameters of a workloads image dict (single block or 'levels' quadtree levels)."""
    from .native import default_params

    levels = int(d.get("levels", 1))
    mb = levels > 1
    return default_params(multiblock=int(mb), max_allowed_level=max(2, levels), dx=d["dx"], edge_fine=int(mb), **kw)


def make_solvers(images, threads=None, **kw):
    """Contexts of the images (workloads dicts), created on all host cores (the
    grid construction is host code called through ctypes).  The plain-cell path
    is fixed to the 8x4 tiles: timing the paths of contexts created at the same
    time would measure them against each other, and every path gives
    bit-identical states."""
    from concurrent.futures import ThreadPoolExecutor

    import torch

    from .native import Solver

    kw.setdefault("plain_path", 2)
    device = torch.cuda.current_device()  # a context lives on its creating thread's current device

    def create(d):
        torch.cuda.set_device(device)
        return Solver(d["pore"], d["kn"], d["locpore"], solver_params(d, **kw))

    with ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 1) as ex:
        return list(ex.map(create, images))


def steady_samples(images, chunk=1000, tol=1e-6, max_steps=100000, log=None):
    """Runs the images (workloads dicts) to steady state as one batch and
    returns (input, target, mask) of those that settled with a positive
    permeability (images of mixed sizes: a list, not an array)."""
    from .native import Batch

    sol = make_solvers(images, concurrent=1)
    b = Batch(sol)
    t0 = time.perf_counter()
    steps, k = run_batch_to_steady(b, chunk=chunk, tol=tol, max_steps=max_steps)
    out = []
    for d, s, st, kk in zip(images, sol, steps, k):
        if st < max_steps and np.isfinite(kk) and kk > 0:
            out.append((network_input(d["pore"], d["kn"]), steady_targets(s), (d["pore"] == 1).astype(np.float32)))
    if log:
        log(f"data: {len(images)} images to steady state in {int(steps.max())} steps "
            f"({time.perf_counter() - t0:.1f} s), kept {len(out)}")
    b.close()
    for s in sol:
        s.close()
    return out


def train_mixed(net, samples, epochs=60, lr=1e-3, pixels_per_batch=8 * 128 * 128, seed=0, log=None):
    """Adam on the masked squared error over samples of mixed sizes: each step
    takes equal-size samples adding up to about pixels_per_batch pixels.
    Returns the mean loss of each epoch."""
    import torch

    rng = np.random.default_rng(seed)
    by_size = {}
    for x, y, m in samples:
        by_size.setdefault(x.shape[-1], []).append((x, encode(y[None], net.scale)[0], m))
    groups = {n: tuple(torch.tensor(np.stack([v[i] for v in vs]), device="cuda") for i in range(3))
              for n, vs in by_size.items()}
    history = []
    t0 = time.perf_counter()
    for ep in range(epochs):
        batches = []
        for n, (X, Y, M) in groups.items():
            per = max(1, pixels_per_batch // (n * n))
            order = rng.permutation(len(X))
            batches += [(n, order[i:i + per]) for i in range(0, len(order), per)]
        rng.shuffle(batches)
        tot, cnt = 0.0, 0
        for n, idx in batches:
            X, Y, M = groups[n]
            sel = torch.tensor(idx, device="cuda")
            x, y, m = X[sel].contiguous(), Y[sel].contiguous(), M[sel].contiguous()
            net.zero_grad()
            p = net.forward(x, keep=True)
            loss, dp = masked_loss(p, y, m)
            net.backward(dp)
            net.adam(lr)
            tot += float(loss.item()) * len(idx)
            cnt += len(idx)
        history.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep + 1}: loss {history[-1]:.4e} ({time.perf_counter() - t0:.1f} s)")
    return history


def smooth_noise(n, seed, passes=8):
    """n x n random field of unit RMS, correlated over a few pixels (neighbour
    averages on the torus)."""
    rng = np.random.default_rng(seed)
    f = rng.standard_normal((n, n))
    for _ in range(passes):
        f = (f + np.roll(f, 1, 0) + np.roll(f, -1, 0) + np.roll(f, 1, 1) + np.roll(f, -1, 1)) / 5.0
    return f / np.sqrt((f * f).mean())


def warm_start_study(net, images, errors=(0.3, 0.1, 0.03, 0.01), blocks=(8, 32, 128), chunk=1000, tol=1e-6,
                     max_steps=200000, log=None):
    """Per held-out image: steps and GPU seconds to the permeability criterion
    (relative change below tol over chunk steps) from rest (cold), from the
    network's prediction (warm: velocity only, and velocity with density), and
    from the converged cold state itself, in parts and with errors put back:
    the exact velocity and density ('exact'), the velocity alone at the rest
    density ('velocity_exact'), the density alone at rest ('density_exact'),
    the exact velocity with the density deviation off by a relative e
    ('density_amplitude_e': (1 + e) drho; 'density_local_e': (1 + e xi) drho, xi
    a smooth unit-RMS random field) or averaged over B x B pixel blocks
    ('density_blocks_B'), and the velocity off by 30 % with the exact density.
    These rows tell which part of a prediction sets the saving and how accurate
    it has to be.  net may be None (the rows without the network)."""
    from .native import Solver

    out = []
    for i, d in enumerate(images):
        p = solver_params(d)
        n = int(d["pore"].shape[0])
        row = {"n": n, "levels": int(d.get("levels", 1)), "kn_mean": d.get("kn_mean")}
        cold = Solver(d["pore"], d["kn"], d["locpore"], p)
        sc, tc, kc = run_to_steady(cold, chunk, tol, max_steps)
        row.update(cold_steps=int(sc), cold_s=tc, k=kc)
        steady = cold.cells()
        px = cold.pixels()
        cx, cy, _ = cold.cell_positions()
        rho_in = cold.info["rho_in"]
        tgt = steady_targets(cold)
        cold.close()
        rest = np.full(steady["ux"].shape, rho_in)
        zero = np.zeros_like(rest)
        drho = steady["rho"] - rho_in

        def restart(rho, ux, uy):
            sv = Solver(d["pore"], d["kn"], d["locpore"], p)
            sv.set_equilibrium(rho, ux, uy)
            st, ts, ks = run_to_steady(sv, chunk, tol, max_steps)
            sv.close()
            return int(st)

        if net is not None:
            for name, dens in (("warm", False), ("warm_density", True)):
                w = Solver(d["pore"], d["kn"], d["locpore"], p)
                t0 = time.perf_counter()
                warm_start(w, net, d["pore"], d["kn"], use_density=dens)
                t_pred = time.perf_counter() - t0
                sw, tw, kw = run_to_steady(w, chunk, tol, max_steps)
                w.close()
                row.update({f"{name}_steps": int(sw), f"{name}_s": tw + t_pred, f"{name}_k_rel": abs(kw - kc) / abs(kc)})
            pred = predict(net, d["pore"], d["kn"])
            void = d["pore"] == 1
            for c, name in ((0, "ux"), (2, "drho")):
                row[f"prediction_rel_err_{name}"] = float(np.abs(pred[c] - tgt[c])[void].mean()
                                                          / max(np.abs(tgt[c])[void].mean(), 1e-30))
        row["exact_steps"] = restart(steady["rho"], steady["ux"], steady["uy"])
        row["velocity_exact_steps"] = restart(rest, steady["ux"], steady["uy"])
        row["density_exact_steps"] = restart(steady["rho"], zero, zero)
        row["velocity_0.3_density_exact_steps"] = restart(steady["rho"], 1.3 * steady["ux"], 1.3 * steady["uy"])
        xi = smooth_noise(n, 7000 + i)[cy, cx]
        for e in errors:
            row[f"density_amplitude_{e:g}_steps"] = restart(rho_in + (1 + e) * drho, steady["ux"], steady["uy"])
            row[f"density_local_{e:g}_steps"] = restart(rho_in + (1 + e * xi) * drho, steady["ux"], steady["uy"])
        void = px["rho"] != 0
        for B in blocks:
            if n % B:
                continue
            # pixel-area mean of the density deviation over B x B blocks (fluid pixels)
            dpx = np.where(void, px["rho"] - rho_in, 0.0)
            num = dpx.reshape(n // B, B, n // B, B).sum(axis=(1, 3))
            den = void.reshape(n // B, B, n // B, B).sum(axis=(1, 3))
            blk = np.where(den > 0, num / np.maximum(den, 1), 0.0)
            coarse = np.kron(blk, np.ones((B, B)))[cy, cx]
            row[f"density_blocks_{B}_steps"] = restart(rho_in + coarse, steady["ux"], steady["uy"])
        # the column and row means of the exact density deviation, and the
        # column model of darcy_column_density
        dpx = np.where(void, px["rho"] - rho_in, 0.0)
        cnt_c = np.maximum(void.sum(axis=0), 1)
        cnt_r = np.maximum(void.sum(axis=1), 1)
        col = np.broadcast_to(dpx.sum(axis=0) / cnt_c, (n, n))[cy, cx]
        rowm = np.broadcast_to((dpx.sum(axis=1) / cnt_r)[:, None], (n, n))[cy, cx]
        row["density_columns_steps"] = restart(rho_in + col, steady["ux"], steady["uy"])
        row["density_rows_steps"] = restart(rho_in + rowm, steady["ux"], steady["uy"])
        model = darcy_column_density(d["pore"], d["locpore"], cold_fbody(p))[cy, cx]
        row["density_column_model_steps"] = restart(rho_in + model, steady["ux"], steady["uy"])
        row["density_column_model_rest_velocity_steps"] = restart(rho_in + model, zero, zero)
        row["column_model_rel_err"] = float(np.abs(model - col).max() / max(np.abs(col).max(), 1e-30))
        # Darcy block models: mobility from the local pore size (H^2), and from the
        # converged velocity (|u| per pixel)
        H = np.asarray(d["locpore"], np.float64)
        speed = np.hypot(px["ux"], px["uy"])
        for B in (16, 32, 64):
            if n % B:
                continue
            for name, mob in (("geometry", H * H), ("speed", speed)):
                dm = darcy_block_density(d["pore"], mob, cold_fbody(p), B)
                row[f"darcy_{name}_{B}_steps"] = restart(rho_in + dm[cy, cx], steady["ux"], steady["uy"])
                blk = dpx.reshape(n // B, B, n // B, B).sum(axis=(1, 3)) / np.maximum(
                    void.reshape(n // B, B, n // B, B).sum(axis=(1, 3)), 1)
                row[f"darcy_{name}_{B}_rel_err"] = float(
                    np.abs(np.where(void, dm - np.kron(blk, np.ones((B, B))), 0.0)).max()
                    / max(np.abs(blk).max(), 1e-30))
        out.append(row)
        if log:
            log(str(row))
    return out


def cold_fbody(p):
    return float(p.fbody)


def darcy_block_density(pore, mobility, fbody, block=32):
    """Density deviation of a Darcy model of the x-periodic image on blocks of
    block x block pixels: block mobility K_b = the mean of `mobility` over the
    block's pixels (solid pixels count 0); between neighbouring blocks the flux
    is T (F B - dp) across x faces (periodic) and -T dp across y faces (none
    through the top and bottom), T the harmonic mean of the two mobilities;
    every block conserves mass.  The scale of the mobility cancels, only its
    variation sets the pressure.  rho - rho_in = 3 p (c_s^2 = 1/3), piecewise
    constant on the blocks, zero mean over the void pixels.  Returns n x n."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.linalg import spsolve

    n = pore.shape[0]
    m = n // block
    void = pore == 1
    mob = np.where(void, np.asarray(mobility, np.float64), 0.0)
    K = mob.reshape(m, block, m, block).mean(axis=(1, 3))
    K = np.maximum(K, 1e-12 * max(K.max(), 1e-300))
    idx = np.arange(m * m).reshape(m, m)  # [row (y), column (x)]
    rows, cols, vals = [], [], []
    rhs = np.zeros(m * m)

    def face(i, j, T, drive):
        # flux from block i to block j: T (drive - (p_j - p_i)); mass balance of both
        rows.extend([i, i, j, j])
        cols.extend([i, j, j, i])
        vals.extend([T, -T, T, -T])
        rhs[i] -= T * drive
        rhs[j] += T * drive

    for y in range(m):
        for x in range(m):
            xr = (x + 1) % m
            Tx = 2 * K[y, x] * K[y, xr] / (K[y, x] + K[y, xr])
            face(idx[y, x], idx[y, xr], Tx, fbody * block)
            if y + 1 < m:
                Ty = 2 * K[y, x] * K[y + 1, x] / (K[y, x] + K[y + 1, x])
                face(idx[y, x], idx[y + 1, x], Ty, 0.0)
    # A p = rhs (flux out minus in); the pressure is fixed up to a constant:
    # pin block 0 and shift afterwards
    A = coo_matrix((vals, (rows, cols)), shape=(m * m, m * m)).tocsr()
    A = A.tolil()
    A[0, :] = 0
    A[0, 0] = 1.0
    rhs[0] = 0.0
    p = spsolve(A.tocsr(), rhs).reshape(m, m)
    drho = 3.0 * np.kron(p, np.ones((block, block)))
    drho = drho - drho[void].mean()
    return np.where(void, drho, 0.0)


def darcy_column_density(pore, locpore, fbody):
    """Density deviation of a Darcy model of the x-periodic pore image, one value
    per column: each column conducts C(x) = sum over its void pixels of H^2
    (H the local pore size, Poiseuille's law), the flux Q is the same through
    every column, so the pressure gradient is dp/dx = F - Q / C(x) with Q set
    by periodicity (the gradients add up to zero over the period); rho - rho_in
    = 3 p (c_s^2 = 1/3), zero mean over the void pixels.  Returns n x n."""
    n = pore.shape[0]
    void = pore == 1
    C = np.where(void, np.asarray(locpore, np.float64) ** 2, 0.0).sum(axis=0)
    inv = np.where(C > 0, 1.0 / np.maximum(C, 1e-300), 0.0)
    g = fbody * (1.0 - inv / inv.mean())   # dp/dx per column, zero mean
    p = np.cumsum(g) - 0.5 * g             # pressure at the column centres
    drho = 3.0 * np.broadcast_to(p, (n, n))
    drho = drho - drho[void].mean()
    return np.where(void, drho, 0.0)


# ---- the coarse density field: the part of the steady state that sets the
# convergence (warm_start_study).  A second network of the same kind works on
# the image coarsened to blocks of COARSE x COARSE pixels, so that its deepest
# features span most of the domain, and predicts the block means of the density
# deviation in units of 3 F n (the pressure a force F builds over the domain).

COARSE = 8


def coarse_input(pore, kn, block=COARSE):
    """2 x n/B x n/B: block porosity and the block mean of log10(Kn) / 2 over void pixels."""
    n = pore.shape[0]
    m = n // block
    void = (pore == 1)
    cnt = void.reshape(m, block, m, block).sum(axis=(1, 3))
    lk = np.where(void, np.log10(np.maximum(kn, 1e-12)) / 2.0, 0.0).reshape(m, block, m, block).sum(axis=(1, 3))
    return np.stack([cnt / float(block * block), np.where(cnt > 0, lk / np.maximum(cnt, 1), 0.0)]).astype(np.float32)


def coarse_density(solver, pore, block=COARSE):
    """1 x n/B x n/B target: block means of rho - rho_in over void pixels, over 3 F n."""
    px = solver.pixels()
    n = pore.shape[0]
    m = n // block
    void = pore == 1
    d = np.where(void, px["rho"] - solver.info["rho_in"], 0.0).reshape(m, block, m, block).sum(axis=(1, 3))
    cnt = void.reshape(m, block, m, block).sum(axis=(1, 3))
    blk = np.where(cnt > 0, d / np.maximum(cnt, 1), 0.0)
    return (blk / (3.0 * solver.params.fbody * n))[None].astype(np.float32)


def coarse_samples(images, chunk=1000, tol=1e-6, max_steps=100000, log=None):
    """(coarse input, coarse density target, block mask) of the images that
    settle with a positive permeability, all stepped as one batch."""
    from .native import Batch

    sol = make_solvers(images, concurrent=1)
    b = Batch(sol)
    t0 = time.perf_counter()
    steps, k = run_batch_to_steady(b, chunk=chunk, tol=tol, max_steps=max_steps)
    out = []
    for d, s, st, kk in zip(images, sol, steps, k):
        if st < max_steps and np.isfinite(kk) and kk > 0:
            x = coarse_input(d["pore"], d["kn"])
            out.append((x, coarse_density(s, d["pore"]), (x[0] > 0).astype(np.float32)))
    if log:
        log(f"coarse data: {len(images)} images in {int(steps.max())} steps ({time.perf_counter() - t0:.1f} s), "
            f"kept {len(out)}")
    b.close()
    for s in sol:
        s.close()
    return out


def augment(samples, rng):
    """x-periodic shifts and y mirror images (symmetries of the flow problem)."""
    out = []
    for x, y, m in samples:
        sh = int(rng.integers(0, x.shape[-1]))
        x, y, m = (np.roll(a, sh, axis=-1) for a in (x, y, m))
        if rng.random() < 0.5:
            x, y, m = x[..., ::-1, :], y[..., ::-1, :], m[..., ::-1, :]
        out.append((np.ascontiguousarray(x), np.ascontiguousarray(y), np.ascontiguousarray(m)))
    return out


def train_coarse(samples, epochs=400, lr=1e-3, widths=(32, 64, 64, 128, 128), seed=0, log=None):
    """The coarse network on augmented samples (a fresh shift and mirror every epoch)."""
    net = UNet(widths=widths, cin=2, cout=1, seed=seed)
    ys = np.concatenate([np.abs(y[0][m > 0]) for _, y, m in samples])
    net.scale = np.array([np.median(ys) + 1e-30])
    rng = np.random.default_rng(seed)
    hist = []
    t0 = time.perf_counter()
    for ep in range(epochs):
        h = train_mixed(net, augment(samples, rng), epochs=1, lr=lr, pixels_per_batch=8 * 64 * 64, seed=ep)
        hist.append(h[0])
        if log and (ep + 1) % 50 == 0:
            log(f"coarse epoch {ep + 1}: loss {hist[-1]:.4e} ({time.perf_counter() - t0:.1f} s)")
    return net, hist


def predict_coarse_density(net, pore, kn, fbody, block=COARSE):
    """n x n density deviation from the coarse network: its block values times
    3 F n, zero mean over the void pixels, 0 on solid pixels."""
    import torch

    n = pore.shape[0]
    x = torch.tensor(coarse_input(pore, kn, block)[None], dtype=torch.float32, device="cuda")
    y = net.forward(x).cpu().numpy()[0, 0].astype(np.float64)
    blk = np.sinh(y) * net.scale[0] * 3.0 * fbody * n
    void = pore == 1
    d = np.kron(blk, np.ones((block, block)))
    d = d - d[void].mean()
    return np.where(void, d, 0.0)


def coarse_study(net, images, chunk=1000, tol=1e-6, max_steps=200000, log=None):
    """Cold start against the coarse network's density (velocity at rest) on
    each image; also the error of the predicted block densities."""
    from .native import Solver

    out = []
    for d in images:
        p = solver_params(d)
        n = d["pore"].shape[0]
        cold = Solver(d["pore"], d["kn"], d["locpore"], p)
        sc, tc, kc = run_to_steady(cold, chunk, tol, max_steps)
        tgt = coarse_density(cold, d["pore"])[0] * 3.0 * p.fbody * n
        cx, cy, _ = cold.cell_positions()
        rho_in = cold.info["rho_in"]
        cold.close()
        pred = predict_coarse_density(net, d["pore"], d["kn"], p.fbody)
        pb = pred.reshape(n // COARSE, COARSE, n // COARSE, COARSE)[:, 0, :, 0]
        mask = coarse_input(d["pore"], d["kn"])[0] > 0
        tb = tgt - tgt[mask].mean()
        err = float(np.abs(pb - tb)[mask].mean() / max(np.abs(tb)[mask].mean(), 1e-30))
        w = Solver(d["pore"], d["kn"], d["locpore"], p)
        t0 = time.perf_counter()
        rho = rho_in + predict_coarse_density(net, d["pore"], d["kn"], p.fbody)[cy, cx]
        w.set_equilibrium(rho, np.zeros_like(rho), np.zeros_like(rho))
        t_pred = time.perf_counter() - t0
        sw, tw, kw = run_to_steady(w, chunk, tol, max_steps)
        w.close()
        row = dict(n=int(n), kn_mean=d.get("kn_mean"), cold_steps=int(sc), cold_s=tc, warm_steps=int(sw),
                   warm_s=tw + t_pred, k_rel=abs(kw - kc) / abs(kc), block_density_rel_err=err)
        out.append(row)
        if log:
            log(str(row))
    return out


def config5(train_images=64, eval_images=4, epochs=60, lr=1e-3, log=None):
    """Trains the network on the steady fields of workloads.config4_steady
    images (sides 128-2048, 1-2 levels) and runs warm_start_study on the
    held-out 1024^2 two-level images workloads.config2_steady(0..eval-1)."""
    from . import workloads

    samples = steady_samples(workloads.generate(workloads.config4_steady, range(train_images)), log=log)
    net = UNet(seed=5)
    ys = [y for _, y, _ in samples]
    ms = [m for _, _, m in samples]
    net.scale = np.array([np.median(np.concatenate([np.abs(y[c][m > 0]) for y, m in zip(ys, ms)])) + 1e-30
                          for c in range(3)])
    t0 = time.perf_counter()
    hist = train_mixed(net, samples, epochs=epochs, lr=lr, log=log)
    t_train = time.perf_counter() - t0
    res = warm_start_study(net, [workloads.config2_steady(i) for i in range(eval_images)], log=log)
    return dict(train_images=len(samples), epochs=epochs, train_seconds=t_train, final_loss=hist[-1],
                first_loss=hist[0], cases=res)


def main(argv=None):
    """python -m mantiis_gb300.surrogate --size 128 --train 512 --epochs 300 --eval 8
    Trains the network on solver-generated steady fields and prints a JSON
    report of the warm start against the cold start."""
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--train", type=int, default=512)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--eval", type=int, default=8)
    ap.add_argument("--lr", type=float, default=5e-4)
    ap.add_argument("--config5", action="store_true",
                    help="train on the config-4 steady set, study the warm start on 1024^2 images")
    ap.add_argument("--coarse", action="store_true",
                    help="train the coarse density network and warm-start the 1024^2 images with its density")
    ap.add_argument("--study-only", action="store_true",
                    help="the warm-start study on the 1024^2 images without training a network")
    a = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)  # noqa: E731
    if a.coarse:
        from . import workloads

        samples = coarse_samples(workloads.generate(workloads.config4_steady, range(a.train))
                                 + workloads.generate(workloads.config2_steady, range(8, 8 + a.train // 2)), log=log)
        net, hist = train_coarse(samples, epochs=a.epochs, lr=a.lr, log=log)
        res = coarse_study(net, [workloads.config2_steady(i) for i in range(a.eval)], log=log)
        print(json.dumps(dict(train_images=len(samples), epochs=a.epochs, first_loss=hist[0], final_loss=hist[-1],
                              cases=res)))
        return
    if a.study_only:
        from . import workloads

        print(json.dumps(warm_start_study(None, [workloads.config2_steady(i) for i in range(a.eval)], log=log)))
        return
    if a.config5:
        print(json.dumps(config5(train_images=a.train, eval_images=a.eval, epochs=a.epochs, lr=a.lr, log=log)))
        return
    X, Y, M = make_dataset(a.size, a.train, log=log)
    net = UNet(seed=1)
    net.scale = target_scale(Y, M)
    t0 = time.perf_counter()
    hist = train(net, X, encode(Y, net.scale), M, epochs=a.epochs, lr=a.lr)
    t_train = time.perf_counter() - t0
    res = evaluate(net, a.size, a.eval, log=log)
    cold = sum(r["cold_steps"] for r in res)
    warm = sum(r["warm_steps"] for r in res)
    print(json.dumps(dict(size=a.size, train_images=len(X), epochs=a.epochs, train_seconds=t_train,
                          final_loss=hist[-1], cold_steps=cold, warm_steps=warm,
                          step_ratio=cold / max(warm, 1), cases=res)))


if __name__ == "__main__":
    main()
