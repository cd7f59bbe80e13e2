"""The warm-start CNN's tensor-core kernels against a PyTorch CPU reference (needs a GPU).

Layer by layer, each GPU result is compared with the reference computed (in
binary64) from the GPU's own input of that layer, so that each check isolates
one kernel:
  forward   bf16(ReLU(conv(X, bf16 W) + b)): every value within one bf16 unit
            in the last place of the reference (or within 1e-5 of the layer's
            largest value, for fp32 accumulation near zero), at least 99%
            identical; last layer x0 + conv + b in fp32: relative L2 <= 1e-5;
  dW, db    sum_v dY[v][co] X[v + tap][ci] from the GPU's bf16 dY and X:
            relative L2 <= 1e-5 (fp32 accumulation);
  dX        (W^T conv dY) masked by X > 0, rounded to bf16: as the forward;
  whole     the GPU's gradients against autograd through the bf16-rounded
            network: cosine similarity >= 0.99 per layer (the GPU rounds
            every dY to bf16, autograd does not).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from pct_gb300 import cnn  # noqa: E402

pytestmark = pytest.mark.gpu

D, H, W = 4, 16, 128
TAPS = 27


def bf16(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(torch.bfloat16).to(torch.float32).numpy()


def conv(x, w, b):
    """x [D, H, W, cin], w [27, cout, cin] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)), b [cout] -> [D, H, W, cout]
    in binary64 with zero padding."""
    cout, cin = w.shape[1], w.shape[2]
    xt = torch.from_numpy(np.ascontiguousarray(x, np.float64)).permute(3, 0, 1, 2).unsqueeze(0)
    wt = torch.from_numpy(np.ascontiguousarray(w, np.float64)).reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)
    y = torch.nn.functional.conv3d(xt, wt, padding=1)[0]
    y = y + torch.from_numpy(np.asarray(b, np.float64))[:, None, None, None]
    return y.permute(1, 2, 3, 0).numpy()


def within_bf16_ulp(gpu, ref):
    r = bf16(ref)
    ulp = np.abs(r) * 2.0 ** -7
    ok = np.abs(gpu - r) <= np.maximum(ulp * 1.001, 1e-5 * np.max(np.abs(ref)))
    same = np.mean(gpu == r)
    return bool(ok.all()) and same >= 0.99, "max excess %.3g, identical %.4f" % (np.max(np.abs(gpu - r) - ulp), same)


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def setup():
    rng = np.random.default_rng(3)
    net = cnn.Net(D, H, W)
    net.init(7)
    p = net.params()
    # non-zero biases and last layer, so that every layer carries gradient
    for k, (ws, shape, bs) in enumerate(cnn.param_slices()):
        p[bs] = rng.uniform(-0.1, 0.1, shape[1]).astype(np.float32)
        if k == len(cnn.LAYERS) - 1:
            p[ws] = rng.uniform(-0.05, 0.05, int(np.prod(shape))).astype(np.float32)
    net.set_params(p)
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    hull = (((xx - 64) ** 2 + (yy - 8) ** 2 * 40) < 50 ** 2).astype(np.uint8)
    x0 = (rng.uniform(0.5, 1.5, (D, H, W)) * hull).astype(np.float32)
    target = (x0 + 0.2 * hull * np.sin(xx / 9.0)).astype(np.float32)
    yield net, p, x0, hull, target
    net.close()


def layer_input(net, x0, hull, l):
    if l == 0:
        x = np.zeros((D, H, W, 2), np.float32)
        x[..., 0] = bf16(x0)
        x[..., 1] = hull
        return x
    return net.inspect(0, l - 1)


def test_forward_every_layer(setup):
    net, p, x0, hull, target = setup
    out = net.forward(x0, hull)
    sl = cnn.param_slices()
    for l in range(7):
        ws, shape, bs = sl[l]
        ref = np.maximum(conv(layer_input(net, x0, hull, l), bf16(p[ws]).reshape(shape), p[bs]), 0.0)
        ok, msg = within_bf16_ulp(net.inspect(0, l), ref)
        assert ok, "layer %d: %s" % (l, msg)
    ws, shape, bs = sl[7]
    ref = x0.astype(np.float64) + conv(net.inspect(0, 6), bf16(p[ws]).reshape(shape), p[bs])[..., 0]
    assert rel_l2(out.reshape(D, H, W), ref) <= 1e-5


def test_gradients_every_layer(setup):
    net, p, x0, hull, target = setup
    out = net.forward(x0, hull).reshape(D, H, W)
    loss, g = net.gradients(x0, hull, target)
    loss2, g2 = net.gradients(x0, hull, target)
    # the CTAs' partial sums meet in float atomics: identical calls agree to rounding
    assert rel_l2(g2, g.astype(np.float64)) <= 1e-6, "gradients of identical calls differ"
    nv = D * H * W
    assert abs(loss - np.mean((out.astype(np.float64) - target) ** 2)) <= 1e-6 * max(loss, 1e-30)
    sl = cnn.param_slices()
    dy7 = net.inspect(1, 7)
    ok, msg = within_bf16_ulp(dy7[..., 0], 2.0 * (out.astype(np.float64) - target) / nv)
    assert ok, "dY7: " + msg
    assert not dy7[..., 1:].any()
    for l in range(8):
        ws, shape, bs = sl[l]
        cout, cin = shape[1], shape[2]
        x = layer_input(net, x0, hull, l)[..., :cin].astype(np.float64)
        dy = (dy7 if l == 7 else net.inspect(1, l))[..., :cout].astype(np.float64)
        xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
        dw = np.empty((TAPS, cout, cin))
        for t in range(TAPS):
            dz, dyy, dx = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
            xs = xp[1 + dz:1 + dz + D, 1 + dyy:1 + dyy + H, 1 + dx:1 + dx + W]
            dw[t] = np.einsum("zyxo,zyxi->oi", dy, xs)
        err = rel_l2(g[ws].reshape(shape), dw)
        assert err <= 1e-5, "dW of layer %d: %.3g" % (l, err)
        assert rel_l2(g[bs], dy.sum(axis=(0, 1, 2))) <= 1e-5, "db of layer %d" % l
        if l > 0:
            # dX = sum over taps of W^T dY shifted back, masked by the layer input > 0
            w = bf16(p[ws]).reshape(shape).astype(np.float64)
            dyp = np.pad(dy, ((1, 1), (1, 1), (1, 1), (0, 0)))
            dxr = np.zeros((D, H, W, cin))
            for t in range(TAPS):
                dz, dyy, dx = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
                dxr += np.einsum("zyxo,oi->zyxi", dyp[1 - dz:1 - dz + D, 1 - dyy:1 - dyy + H, 1 - dx:1 - dx + W], w[t])
            dxr *= layer_input(net, x0, hull, l)[..., :cin] > 0
            ok, msg = within_bf16_ulp(net.inspect(1, l - 1), dxr)
            assert ok, "dY of layer %d: %s" % (l - 1, msg)


def test_whole_backward_matches_autograd(setup):
    net, p, x0, hull, target = setup
    loss, g = net.gradients(x0, hull, target)
    sl = cnn.param_slices()
    params = [torch.tensor(bf16(p[ws]).reshape(shape), dtype=torch.float64, requires_grad=True) for ws, shape, _ in sl]
    biases = [torch.tensor(p[bs], dtype=torch.float64, requires_grad=True) for _, _, bs in sl]
    x = torch.zeros((1, 2, D, H, W), dtype=torch.float64)
    x[0, 0] = torch.from_numpy(bf16(x0).astype(np.float64))
    x[0, 1] = torch.from_numpy(hull.astype(np.float64))
    a = x
    for l, (w, b) in enumerate(zip(params, biases)):
        cout, cin = w.shape[1], w.shape[2]
        wt = w.reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)
        a = torch.nn.functional.conv3d(a, wt, padding=1) + b[:, None, None, None]
        if l < 7:
            a = torch.relu(a)
            a = a + (a.detach().float().to(torch.bfloat16).double() - a.detach())  # bf16 forward, straight-through
    out = torch.from_numpy(x0.astype(np.float64)) + a[0, 0]
    lt = torch.mean((out - torch.from_numpy(target.astype(np.float64))) ** 2)
    lt.backward()
    for l, (ws, shape, bs) in enumerate(sl):
        ref = params[l].grad.numpy().ravel()
        cos = float(np.dot(g[ws], ref) / (np.linalg.norm(g[ws]) * np.linalg.norm(ref) + 1e-300))
        assert cos >= 0.99, "layer %d: cosine %.4f" % (l, cos)
    assert abs(loss - lt.item()) <= 1e-3 * lt.item()


def test_adam_steps_reduce_the_loss():
    rng = np.random.default_rng(5)
    net = cnn.Net(D, H, W)
    net.init(11)
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    hull = (np.abs(xx - 64) < 48).astype(np.uint8)
    x0 = (rng.uniform(0.8, 1.2, (D, H, W)) * hull).astype(np.float32)
    target = (0.5 * x0 + 0.3 * hull).astype(np.float32)
    losses = [net.train_step(x0, hull, target, 2e-3) for _ in range(150)]
    net.close()
    assert losses[-1] < 0.1 * losses[0], losses[::25]


def test_weight_gradients_with_many_chunks_per_cta():
    """At 8 x 64 x 128 voxels each CTA of the weight-gradient kernel accumulates 14
    voxel chunks through its 3-stage ring (the small volume above gives 2): the
    weight and bias gradients of a hidden layer against binary64."""
    d, h = 8, 64
    rng = np.random.default_rng(9)
    net = cnn.Net(d, h, W)
    net.init(4)
    p = net.params()
    sl = cnn.param_slices()
    for k, (ws, shape, bs) in enumerate(sl):
        p[bs] = rng.uniform(-0.1, 0.1, shape[1]).astype(np.float32)
        if k == len(cnn.LAYERS) - 1:
            p[ws] = rng.uniform(-0.05, 0.05, int(np.prod(shape))).astype(np.float32)
    net.set_params(p)
    zz, yy, xx = np.meshgrid(np.arange(d), np.arange(h), np.arange(W), indexing="ij")
    hull = (((xx - 64) ** 2 + (yy - 32) ** 2) < 50 ** 2).astype(np.uint8)
    x0 = (rng.uniform(0.5, 1.5, (d, h, W)) * hull).astype(np.float32)
    target = (x0 + 0.2 * hull * np.cos(yy / 7.0)).astype(np.float32)
    loss, g = net.gradients(x0, hull, target)
    for l in (3, 7):
        ws, shape, bs = sl[l]
        cout, cin = shape[1], shape[2]
        x = net.inspect(0, l - 1)[..., :cin].astype(np.float64).reshape(d, h, W, cin)
        dy = net.inspect(1, l)[..., :cout].astype(np.float64).reshape(d, h, W, -1)[..., :cout]
        xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
        dw = np.empty((TAPS, cout, cin))
        for t in range(TAPS):
            dz, dyy, dx = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
            xs = xp[1 + dz:1 + dz + d, 1 + dyy:1 + dyy + h, 1 + dx:1 + dx + W]
            dw[t] = np.einsum("zyxo,zyxi->oi", dy, xs)
        err = rel_l2(g[ws].reshape(shape), dw)
        assert err <= 1e-5, "dW of layer %d: %.3g" % (l, err)
        assert rel_l2(g[bs], dy.sum(axis=(0, 1, 2))) <= 1e-5, "db of layer %d" % l
    net.close()
