"""The warm-start network's GPU kernels (libmantiis_cnn.so) against the FP64
oracle (oracle/cnn_oracle.py): forward output, loss and every layer's weight
and bias gradients, on a narrow network so that the oracle runs in seconds;
and one Adam step with its BF16 copy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16_to_float(t16):
    u = t16.cpu().numpy().view(np.uint16).astype(np.uint32) << 16
    return u.view(np.float32).astype(np.float64)


def test_network_gradients_match_oracle():
    import torch

    from mantiis_gb300 import surrogate as S
    from oracle import cnn_oracle as co

    net = S.UNet(widths=(8, 8, 16, 16, 16), seed=3)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((2, 2, 32, 32)).astype(np.float32)
    t = rng.standard_normal((2, 3, 32, 32)).astype(np.float32)
    mask = (rng.random((2, 32, 32)) > 0.3).astype(np.float32)
    X, T, M = (torch.tensor(a, device="cuda") for a in (x, t, mask))
    net.zero_grad()
    p = net.forward(X, keep=True)
    loss, dp = S.masked_loss(p, T, M)
    net.backward(dp)
    torch.cuda.synchronize()
    params = [(bf16_to_float(l.w16).reshape(l.w.shape), l.b.cpu().numpy()) for l in net.layers()]
    ref = co.Net(params)
    yref = ref.forward(x.astype(np.float64))
    lref, dref = co.masked_loss(yref, t, mask)
    grads = ref.backward(dref)
    # FP32 activations against FP64: relative bounds
    e_y = np.abs(p.cpu().numpy() - yref).max() / np.abs(yref).max()
    assert e_y < 1e-5
    assert abs(float(loss.item()) - lref) < 1e-5 * lref
    for l, (gw, gb) in zip(net.layers(), grads):
        e_w = np.abs(l.dw.cpu().numpy() - gw).max() / max(np.abs(gw).max(), 1e-30)
        e_b = np.abs(l.db.cpu().numpy() - gb).max() / max(np.abs(gb).max(), 1e-30)
        assert e_w < 1e-4 and e_b < 1e-4, (e_w, e_b)


def test_adam_step_and_bf16_copy():
    import torch

    from mantiis_gb300 import surrogate as S

    rng = np.random.default_rng(1)
    layer = S.Conv3x3(4, 4, rng)
    w0 = layer.w.cpu().numpy().copy()
    g = rng.standard_normal(w0.shape).astype(np.float32)
    layer.dw.copy_(torch.tensor(g, device="cuda"))
    layer.adam(1e-2, 1)
    torch.cuda.synchronize()
    # first Adam step: w - lr * g / (|g| + eps)
    expect = w0 - 1e-2 * g / (np.abs(g) + 1e-8)
    assert np.abs(layer.w.cpu().numpy() - expect).max() < 1e-6
    w16 = bf16_to_float(layer.w16).reshape(w0.shape)
    assert np.abs(w16 - layer.w.cpu().numpy()).max() <= np.abs(layer.w.cpu().numpy()).max() * 2 ** -8


def test_train_and_warm_start_small():
    # the whole loop on a small case: solver-made training data, training on
    # the GPU kernels, then the warm-started solver converges to the cold
    # start's permeability; the step counts of both are recorded.  The network
    # predicts the velocity well enough to look right but saves no steps (on
    # one of these images it costs 1000 more): the slow part of the convergence
    # is the density field (test_warm_start_needs_the_density)
    from mantiis_gb300 import surrogate as S
    from test_gpu_transport import record

    X, Y, M = S.make_dataset(64, 32, chunk=250, tol=1e-6, max_steps=20000)
    assert len(X) >= 24
    net = S.UNet(widths=(16, 32, 64, 64, 64), seed=2)
    net.scale = S.target_scale(Y, M)
    hist = S.train(net, X, S.encode(Y, net.scale), M, epochs=150, batch=8, lr=2e-3)
    assert min(hist[-10:]) < 0.25 * hist[0]
    # a criterion tight enough that both runs settle within 1e-5 of each other
    res = S.evaluate(net, 64, 2, chunk=250, tol=1e-8, max_steps=80000)
    for i, r in enumerate(res):
        assert r["warm_steps"] < 80000 and r["cold_steps"] < 80000
        assert r["permeability_rel_diff"] < 1e-5
        record(f"warm_start_64_{i}", cold_steps=r["cold_steps"], warm_steps=r["warm_steps"],
               prediction_rel_err=r["prediction_rel_err"], k_rel=r["permeability_rel_diff"])


def test_warm_start_needs_the_density():
    # What a warm start has to get right: restarting from the converged state
    # itself reaches the criterion in far fewer steps than the cold start, but
    # the converged velocity alone, at the rest density, saves nothing -- the
    # slow part of the convergence is the density (pressure) field
    from mantiis_gb300 import Solver
    from mantiis_gb300 import surrogate as S
    from test_gpu_transport import record

    from mantiis_gb300 import workloads

    # a 1024^2 two-level image whose cold start is slow (117k steps)
    d = workloads.config2_steady(3)
    p = S.solver_params(d)
    chunk, tol = 1000, 1e-6
    cold = Solver(d["pore"], d["kn"], d["locpore"], p)
    sc, _, kc = S.run_to_steady(cold, chunk, tol, 200000)
    st = cold.cells()
    rho_in = cold.info["rho_in"]
    cold.close()

    def restart(rho, ux, uy):
        s = Solver(d["pore"], d["kn"], d["locpore"], p)
        s.set_equilibrium(rho, ux, uy)
        n, _, k = S.run_to_steady(s, chunk, tol, 200000)
        s.close()
        assert abs(k - kc) < 1e-5 * abs(kc)
        return n

    exact = restart(st["rho"], st["ux"], st["uy"])
    velocity_only = restart(np.full_like(st["rho"], rho_in), st["ux"], st["uy"])
    record("warm_start_needs_density_1024", cold_steps=sc, exact_steps=exact, velocity_only_steps=velocity_only)
    # measured on a GB300: cold 117000, exact 6000, velocity only 117000
    assert sc < 200000
    assert exact <= 0.2 * sc
    assert velocity_only >= 0.9 * sc


def test_settled_images_leave_the_batch():
    # six small config-4 steady images (sides 128 / 256) run to steady state
    # twice: once with every image stepped to the end, once with each image
    # leaving the batch when it settles.  An image's arithmetic does not depend
    # on the batch around it, so both runs see every image settle at the same
    # step, with the same permeability then; dropping them saves lattice updates
    from mantiis_gb300 import Batch, Solver, workloads
    from mantiis_gb300.surrogate import run_batch_to_steady, solver_params

    imgs = [workloads.config4_steady(i) for i in (5, 6, 9, 10, 11, 12)]
    out = {}
    for drop in (False, True):
        sol = [Solver(d["pore"], d["kn"], d["locpore"], solver_params(d, concurrent=1)) for d in imgs]
        b = Batch(sol)
        stats = {}
        steps, k = run_batch_to_steady(b, chunk=1000, tol=1e-6, max_steps=60000, drop_settled=drop, stats=stats)
        k_settled = np.array([s.observables()["permeability"] for s in sol])
        out[drop] = (steps, k, k_settled, stats)
        b.close()
        for s in sol:
            s.close()
    (st0, k0, _, s0), (st1, k1, ks1, s1) = out[False], out[True]
    assert np.array_equal(st0, st1)
    assert (st1 < 60000).sum() >= 4
    settled = st1 < 60000
    # dropped images hold their state at the settling step: the returned k is
    # theirs (FP64 atomic sums: equal to 1e-12)
    assert np.allclose(k1[settled], ks1[settled], rtol=1e-12, atol=0)
    # stepped on, a settled image's permeability moves by less than the criterion per chunk
    extra = (st0.max() - st1[settled]) / 1000.0
    assert np.all(np.abs(k0[settled] - k1[settled]) <= 1e-6 * np.abs(k1[settled]) * (extra + 1))
    assert s1["lu"] < s0["lu"] and s1["batches"] > 1
