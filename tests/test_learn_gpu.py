"""The learned active-set warm start: the MLP's hand-written forward and
backward kernels against an FP64 CPU restatement of the same network (the
BF16-rounded weights it computes with, ReLU hidden layers, weighted sigmoid
cross-entropy), training, and what the trained model gains over cold starts
on a parametric MPC family (fresh theta): every solve Optimal at eps_abs =
1e-8 with the same solution, fewer active-set iterations."""
import numpy as np
import pytest

import nasoq_gb300 as nq
from nasoq_gb300 import problems as P


def bf16_round(a):
    """Round-to-nearest-even of float32 values to bfloat16, returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def cpu_loss_grad(layers, x, y, pw):
    """FP64 forward / backward of the MLP (layers: [(W_bf16, b)])."""
    acts = [x.astype(np.float64)]
    L = len(layers)
    for l, (W, b) in enumerate(layers):
        z = acts[-1] @ W.astype(np.float64).T + b.astype(np.float64)
        acts.append(np.maximum(z, 0.0) if l + 1 < L else z)
    z = acts[-1]
    s = 1.0 / (1.0 + np.exp(-z))
    M = x.shape[0]
    sp_neg = np.maximum(-z, 0) + np.log1p(np.exp(-np.abs(z)))
    sp_pos = np.maximum(z, 0) + np.log1p(np.exp(-np.abs(z)))
    loss = (pw * y * sp_neg + (1 - y) * sp_pos).sum() / M
    d = (s * (pw * y + 1 - y) - pw * y) / M
    gws, gbs = [None] * L, [None] * L
    for l in range(L - 1, -1, -1):
        W = layers[l][0].astype(np.float64)
        gws[l] = d.T @ acts[l]
        gbs[l] = d.sum(axis=0)
        if l > 0:
            d = (d @ W) * (acts[l] > 0)
    return loss, np.concatenate([g.ravel() for g in gws]), np.concatenate(gbs)


@pytest.mark.gpu
def test_mlp_gradients_match_cpu_fp64():
    sizes = (32, 48, 40, 70)
    m = nq.MLP(sizes, seed=3)
    rng = np.random.default_rng(4)
    w, b = m.get_weights()
    b = rng.normal(0, 0.1, b.shape).astype(np.float32)
    m.set_weights(w, b)
    x = rng.standard_normal((257, sizes[0])).astype(np.float32)
    y = (rng.random((257, sizes[-1])) < 0.15).astype(np.float32)
    loss, gw, gb = m.loss_grad(x, y, pos_weight=4.0)
    layers = [(bf16_round(W), bb) for W, bb in m.layers()]
    cl, cgw, cgb = cpu_loss_grad(layers, x, y, 4.0)
    assert abs(loss - cl) <= 1e-5 * abs(cl)
    assert np.abs(gw - cgw).max() <= 1e-4 * np.abs(cgw).max()
    assert np.abs(gb - cgb).max() <= 1e-4 * np.abs(cgb).max()
    # the forward pass alone: logits of the CPU network
    z = m.forward(x)
    a = x.astype(np.float64)
    for l, (W, bb) in enumerate(layers):
        a = a @ W.astype(np.float64).T + bb
        if l + 1 < len(layers):
            a = np.maximum(a, 0)
    assert np.abs(z - a).max() <= 1e-4 * np.abs(a).max()
    m.close()


@pytest.mark.gpu
def test_mlp_training_reduces_loss():
    rng = np.random.default_rng(5)
    x = rng.standard_normal((4096, 16)).astype(np.float32)
    y = (x[:, :8] + 0.3 * x[:, 8:] > 0.5).astype(np.float32)  # a learnable rule
    m = nq.MLP((16, 64, 8), seed=1)
    losses = m.fit(x, y, epochs=15, batch=256, lr=3e-3, pos_weight=1.0, seed=2)
    assert losses[-1] < 0.5 * losses[0]
    m.close()


@pytest.mark.gpu
def test_learned_warm_start_gains_over_cold_start():
    pytest.importorskip("torch")
    from nasoq_gb300 import learn

    fam = P.mpc_parametric(0)
    model, rep = learn.train_model(fam, n_train=8192, seed=11, epochs=30, batch=512, lr=2e-3,
                                   solver=dict(variant=0, eps_abs=1e-8))
    assert rep.losses[-1] < rep.losses[0]
    n_eval = 1024
    thetas = np.random.default_rng(999).standard_normal((n_eval, fam.P.shape[1]))
    batch = learn.family_batch(fam, n_eval, variant=0, eps_abs=1e-8, precision=nq.NQG_FP32, refine=1,
                               refine_tol=1e-12)
    ws = learn.WarmStarter(batch, model, fam)
    xc, _, zc, sc = ws.solve(thetas, warm=False)
    xw, _, zw, sw = ws.solve(thetas, warm=True)
    cold_it = np.array([s.num_iter for s in sc])
    warm_it = np.array([s.num_iter for s in sw])
    assert all(s.status == 1 for s in sc) and all(s.status == 1 for s in sw)
    assert all(s.lag_res <= 1e-8 and s.cons_sat_norm <= 1e-8 for s in sw)
    n = fam.base.n
    err = np.abs(xw - xc).reshape(n_eval, n).max(axis=1) / np.maximum(np.abs(xc).reshape(n_eval, n).max(axis=1), 1)
    assert err.max() <= 1e-6
    print(f"iterations: cold {cold_it.mean():.2f}, warm {warm_it.mean():.2f} per problem")
    assert warm_it.mean() <= 0.75 * cold_it.mean()
    batch.close()
    model.close()
