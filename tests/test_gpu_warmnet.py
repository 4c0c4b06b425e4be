"""The learned warm-start net's BF16 tensor-core kernels against a plain
PyTorch float64 restatement of the same net (tests/warmnet_torch.py).

Tolerances: the native path rounds every activation and gradient to BF16
(8 significant bits) between layers, the reference keeps float64 after
rounding only the weights and input features to BF16.  Output: normwise
relative error <= 3e-2.  Loss: relative error <= 3e-2.  Parameter gradients,
per layer: normwise relative error <= 6e-2 and cosine similarity >= 0.998."""
import numpy as np
import pytest
import torch

import warmnet_torch as wt

pytestmark = pytest.mark.gpu


def _lattice(qmin, seed, side):
    from importlib import import_module
    w = import_module("qmin_gb300.workloads")
    return w.c4_solve(seed, side=side)


def _dev(sol):
    n = sol["Q"].shape[0]
    q = torch.as_tensor(np.ascontiguousarray(sol["Q"].T)).cuda()  # SoA planes, stride n
    t = torch.as_tensor(sol["types"].astype(np.int8)).cuda()
    return q, t, n


def _features_numpy(sol):
    Q, types, objs = sol["Q"], sol["types"], sol["objects"]
    n = Q.shape[0]
    f = np.zeros((n, 16), dtype=np.float32)
    f[:, :5] = Q
    obj = types > 0
    f[obj, 5] = 1.0
    f[types == -1, 6] = 1.0
    for j, (kind, W, _S0) in enumerate(objs):
        sel = types == j + 1
        f[sel, 7] = np.float32(0.1) * np.float32(W)
        f[sel, 8] = 1.0 if kind == 0 else 0.0
        f[sel, 9] = 1.0 if kind == 1 else 0.0
    return wt.bf16_round(f).numpy(), (types <= 0).astype(np.uint8)


def _net_with_inputs(qmin, sols, train=True, seed=3, head_scale=1.0):
    L = sols[0]["L"]
    net = qmin.WarmNet(len(sols), L, train=train)
    net.set_params(qmin.warmnet_init_params(seed, head_scale=head_scale))
    keep = []
    for k, s in enumerate(sols):
        q, t, n = _dev(s)
        keep.append((q, t))
        torch.cuda.synchronize()
        net.features(k, q.data_ptr(), qmin.FP64, n, t.data_ptr(), s["objects"])
    net.sync()
    return net, keep


def test_features_match_definition(qmin):
    sols = [_lattice(qmin, 11, 16), _lattice(qmin, 12, 16)]
    net, _keep = _net_with_inputs(qmin, sols, train=False)
    x, _y, m = net.torch_views()
    xs = x.float().cpu().numpy()
    ms = m.cpu().numpy()
    for k, s in enumerate(sols):
        fx, fm = _features_numpy(s)
        assert np.array_equal(xs[k], fx)
        assert np.array_equal(ms[k], fm)


@pytest.mark.parametrize("L", [(16, 16, 16), (24, 8, 16)])
def test_forward_matches_torch_fp64(qmin, L):
    sols = []
    for seed in (21, 22):
        s = _lattice(qmin, seed, max(L))
        if L != (max(L),) * 3:
            # a non-cubic lattice: crop the cube's arrays to L (types stay valid labels)
            side = max(L)
            idx = np.arange(side ** 3).reshape(side, side, side)[:L[2], :L[1], :L[0]].ravel()
            s = dict(s, L=L, Q=np.ascontiguousarray(s["Q"][idx]), types=np.ascontiguousarray(s["types"][idx]))
        sols.append(s)
    net, _keep = _net_with_inputs(qmin, sols, train=False)
    net.forward()
    net.sync()
    x, y, _m = net.torch_views()
    yg = y.cpu().numpy().astype(np.float64)
    xs = x.float().cpu().numpy()
    p = net.get_params()
    P = wt.unpack(p, qmin.WARMNET_LAYERS)
    B, n = len(sols), L[0] * L[1] * L[2]
    xt = torch.as_tensor(xs.astype(np.float64)).reshape(B, L[2], L[1], L[0], 16).permute(0, 4, 1, 2, 3)
    with torch.no_grad():
        yr = wt.forward(P, xt).permute(0, 2, 3, 4, 1).reshape(B, n, 16).numpy()
    err = np.linalg.norm(yg - yr) / np.linalg.norm(yr)
    assert err <= 3e-2, err


@pytest.mark.parametrize("L", [(16, 16, 16), (24, 8, 16)])
def test_tcgen05_matches_mma_sync(qmin, L):
    """The tcgen05 convolutions (tensor-memory accumulators) against the
    mma.sync ones on the same BF16 operands: every layer's output agrees to
    FP32 accumulation order and the BF16 rounding of the activations between
    layers (final output normwise relative difference <= 1e-2), the loss to
    1e-2 and every parameter gradient to 2e-2."""
    sols = []
    for seed in (71, 72):
        s = _lattice(qmin, seed, max(L))
        if L != (max(L),) * 3:
            side = max(L)
            idx = np.arange(side ** 3).reshape(side, side, side)[:L[2], :L[1], :L[0]].ravel()
            s = dict(s, L=L, Q=np.ascontiguousarray(s["Q"][idx]), types=np.ascontiguousarray(s["types"][idx]))
        sols.append(s)
    rng = np.random.default_rng(9)
    n = L[0] * L[1] * L[2]
    tgt = torch.as_tensor((0.3 * rng.standard_normal((2, n, 5))).astype(np.float32)).cuda()
    outs = []
    for tc in (False, True):
        net, _keep = _net_with_inputs(qmin, sols, train=True)
        net.set_tensor_path(tc)
        net.forward()
        torch.cuda.synchronize()
        loss = net.backward(tgt.data_ptr())
        net.sync()
        _x, y, _m = net.torch_views()
        outs.append((y.float().cpu().numpy().astype(np.float64), loss, net.get_params(grads=True)[1]))
    (y0, l0, g0), (y1, l1, g1) = outs
    assert np.isfinite(y1).all()
    assert np.linalg.norm(y1 - y0) <= 1e-2 * np.linalg.norm(y0)
    assert abs(l1 - l0) <= 1e-2 * abs(l0)
    assert np.linalg.norm(g1 - g0) <= 2e-2 * np.linalg.norm(g0)


@pytest.mark.parametrize("L", [(40, 48, 24), (56, 40, 16)])
def test_tma_staging_matches_thread_staging(qmin, L):
    """The direct 3^3 kernel with its halo planes staged by TMA (tensor path
    1, the default) against the same kernel staged by the threads (path 2):
    the MMAs read the same operands in the same order, so the outputs are
    identical bit for bit (the loss and the gradients to their atomic
    summation order).  Two samples (the tensor
    map's sample coordinate), tiles that overhang the grid in x and y (56 x 40:
    16-row tiles over 40 rows, 8-wide tiles over 28 columns at level 1), and
    the zero padding read past every face."""
    sols = []
    for seed in (81, 82):
        s = _lattice(qmin, seed, max(L))
        side = max(L)
        idx = np.arange(side ** 3).reshape(side, side, side)[:L[2], :L[1], :L[0]].ravel()
        sols.append(dict(s, L=L, Q=np.ascontiguousarray(s["Q"][idx]), types=np.ascontiguousarray(s["types"][idx])))
    rng = np.random.default_rng(11)
    n = L[0] * L[1] * L[2]
    tgt = torch.as_tensor((0.3 * rng.standard_normal((2, n, 5))).astype(np.float32)).cuda()
    outs = []
    for path in (2, 1):
        net, _keep = _net_with_inputs(qmin, sols, train=True)
        net.set_tensor_path(path)
        net.forward()
        torch.cuda.synchronize()
        loss = net.backward(tgt.data_ptr())
        net.sync()
        _x, y, _m = net.torch_views()
        outs.append((y.float().cpu().numpy(), loss, net.get_params(grads=True)[1]))
        net.close()
    (y0, l0, g0), (y1, l1, g1) = outs
    assert np.isfinite(y1).all()
    assert np.array_equal(y0, y1)
    # the loss and the weight gradients are summed with atomics (their order varies run to run)
    assert abs(l1 - l0) <= 1e-12 * abs(l0)
    assert np.linalg.norm(g1 - g0) <= 1e-5 * np.linalg.norm(g0)


def test_tma_wait_limit_reports_and_recovers(qmin):
    """The TMA direct convolution's bounded waits made to run out: with a poll
    limit of zero every CTA gives up at its first wait, lets the copies it
    issued land, frees its tensor memory and raises the device error word;
    the pass then reports QMIN_ETIMEOUT through sync.  With the default limit
    restored the same net's next pass is identical to a clean one."""
    L = (40, 48, 24)
    side = max(L)
    s = _lattice(qmin, 91, side)
    idx = np.arange(side ** 3).reshape(side, side, side)[:L[2], :L[1], :L[0]].ravel()
    sols = [dict(s, L=L, Q=np.ascontiguousarray(s["Q"][idx]), types=np.ascontiguousarray(s["types"][idx]))]
    net, _keep = _net_with_inputs(qmin, sols, train=False)
    net.set_tensor_path(1)
    _x, y, _m = net.torch_views()
    net.forward()
    net.sync()
    y_ref = y.float().cpu().numpy().copy()
    try:
        qmin.set_wait_limit(0)
        net.forward()
        with pytest.raises(qmin.QminError) as err:
            net.sync()
        assert err.value.code == qmin.QMIN_ETIMEOUT
        assert "gave up" in str(err.value)
    finally:
        qmin.set_wait_limit(-1)
    net.forward()
    net.sync()
    assert np.array_equal(y.float().cpu().numpy(), y_ref)
    net.close()


def test_backward_matches_torch_fp64(qmin):
    L = (16, 16, 16)
    sols = [_lattice(qmin, s, 16) for s in (31, 32)]
    net, _keep = _net_with_inputs(qmin, sols, train=True)
    rng = np.random.default_rng(5)
    n = 16 ** 3
    target = (0.3 * rng.standard_normal((2, n, 5))).astype(np.float32)
    tgt = torch.as_tensor(target).cuda()
    net.forward()
    torch.cuda.synchronize()
    loss = net.backward(tgt.data_ptr())
    p, g = net.get_params(grads=True)
    x, _y, m = net.torch_views()
    xs = x.float().cpu().numpy()
    ms = m.cpu().numpy()
    _yr, loss_r, g_r = wt.loss_and_grads(p, qmin.WARMNET_LAYERS, xs, target, ms, L)
    assert abs(loss - loss_r) <= 3e-2 * loss_r, (loss, loss_r)
    for i, (ws, bs, spec) in enumerate(qmin.warmnet_param_slices()):
        for sl, what in ((ws, "w"), (bs, "b")):
            a, b = g[sl].astype(np.float64), g_r[sl]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            cos = float(a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30))
            assert rel <= 6e-2 and cos >= 0.998, (i, what, spec, rel, cos)


def test_adam_steps_reduce_loss(qmin):
    sols = [_lattice(qmin, s, 16) for s in (41, 42)]
    net, _keep = _net_with_inputs(qmin, sols, train=True, head_scale=0.1)
    # target: the initial Q smoothed over the six neighbours
    tg = []
    for s in sols:
        q = s["Q"].reshape(16, 16, 16, 5)
        sm = sum(np.roll(q, sh, ax) for ax in (0, 1, 2) for sh in (1, -1)) / 6.0
        tg.append(sm.reshape(-1, 5))
    tgt = torch.as_tensor(np.array(tg, dtype=np.float32)).cuda()
    torch.cuda.synchronize()
    losses = []
    for it in range(40):
        net.forward()
        losses.append(net.backward(tgt.data_ptr()))
        net.adam_step(2e-3)
    assert losses[-1] < 0.5 * losses[0], losses[::8]


def test_warm_start_writes_only_moved_sites(qmin):
    s = _lattice(qmin, 51, 16)
    for prec in (qmin.FP64, qmin.FP32):
        lat = qmin.Lattice(s["L"], prec)
        a, b, c = s["consts"]
        lat.set_params(a, b, c, *s["Ls"])
        lat.set_objects(s["objects"])
        lat.set_state(s["Q"], s["types"])
        net = qmin.WarmNet(1, s["L"])
        net.set_params(qmin.warmnet_init_params(7, head_scale=1.0))
        lat.warm_start(net)
        q = lat.get_state()[0]
        _x, y, _m = net.torch_views()
        yp = y[0, :, :5].cpu().numpy().astype(np.float64)
        obj = s["types"] > 0
        q0 = s["Q"] if prec == qmin.FP64 else s["Q"].astype(np.float32).astype(np.float64)
        assert np.array_equal(q[obj], q0[obj])
        want = yp[~obj] if prec == qmin.FP64 else yp[~obj].astype(np.float32).astype(np.float64)
        assert np.array_equal(q[~obj], want)
        assert net.launches() > 0
        # FIRE runs from the warm-started state
        lat.fire_init()
        r = lat.fire_run(5)
        assert np.isfinite(r["forceMax"])


def test_warm_start_rejects_mismatched_net(qmin):
    s = _lattice(qmin, 61, 16)
    lat = qmin.Lattice(s["L"])
    a, b, c = s["consts"]
    lat.set_params(a, b, c, *s["Ls"])
    lat.set_objects(s["objects"])
    lat.set_state(s["Q"], s["types"])
    net = qmin.WarmNet(1, (16, 16, 8))
    with pytest.raises(qmin.QminError):
        lat.warm_start(net)
    inf = qmin.WarmNet(1, (16, 16, 16), train=False)
    tgt = torch.zeros((16 ** 3, 5), dtype=torch.float32, device="cuda")
    with pytest.raises(qmin.QminError) as e:
        inf.backward(tgt.data_ptr())
    assert e.value.code == 4
