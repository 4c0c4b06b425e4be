"""Plain PyTorch (CPU, float64) restatement of the learned warm-start net, for
checking the native BF16 tensor-core kernels: the same layers, parameter
layout and masked loss as the native library.  Test infrastructure only."""
import numpy as np
import torch
import torch.nn.functional as Fn


def bf16_round(a):
    """Round float32 values to bfloat16 (round to nearest even), as float64."""
    t = torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32))
    return t.to(torch.bfloat16).to(torch.float64)


def unpack(params, layers, bf16_weights=True):
    """Torch conv3d weights [cout, cin, kz, ky, kx] and biases from the flat
    vector (weights stored [cout][tap][cin], tap = kx + 3 ky + 9 kz)."""
    out, off = [], 0
    for (cin, cout, taps, stride, _lvl, relu) in layers:
        w = params[off:off + cout * taps * cin]
        off += cout * taps * cin
        b = params[off:off + cout]
        off += cout
        wt = bf16_round(w) if bf16_weights else torch.as_tensor(np.asarray(w, dtype=np.float64))
        k = 3 if taps == 27 else 1
        wt = wt.reshape(cout, k, k, k, cin).permute(0, 4, 1, 2, 3).contiguous()
        out.append(dict(w=wt.requires_grad_(True), b=torch.as_tensor(np.asarray(b, dtype=np.float64)).requires_grad_(True),
                        stride=stride, pad=1 if taps == 27 else 0, relu=relu))
    return out


def forward(P, x):
    """x: [B, 16, z, y, x] float64 -> y [B, 16, z, y, x]."""
    def conv(i, h):
        p = P[i]
        o = Fn.conv3d(h, p["w"], p["b"], stride=p["stride"], padding=p["pad"])
        return torch.relu(o) if p["relu"] else o

    up = lambda h: Fn.interpolate(h, scale_factor=2, mode="nearest")  # noqa: E731
    a0 = conv(0, x)
    a1 = conv(1, a0)
    a2 = conv(2, a1)
    a3 = conv(3, a2)
    a4 = up(conv(4, a3)) + a2
    a5 = conv(5, a4)
    a6 = up(conv(6, a5)) + a1
    a7 = conv(7, a6)
    a8 = up(conv(8, a7)) + a0
    a9 = conv(9, a8)
    return conv(10, a9)


def grads_flat(P):
    """Gradients in the flat-vector layout ([cout][tap][cin] weights, biases)."""
    parts = []
    for p in P:
        g = p["w"].grad.permute(0, 2, 3, 4, 1).reshape(-1)
        parts.append(g)
        parts.append(p["b"].grad.reshape(-1))
    return torch.cat(parts).numpy()


def loss_and_grads(params, layers, x_sites, target, mask, L):
    """x_sites [B, sites, 16], target [B, sites, 5], mask [B, sites] (numpy);
    returns (y [B, sites, 16], loss, flat gradients)."""
    Lx, Ly, Lz = L
    B = x_sites.shape[0]
    P = unpack(params, layers)
    x = torch.as_tensor(np.asarray(x_sites, dtype=np.float64)).reshape(B, Lz, Ly, Lx, 16).permute(0, 4, 1, 2, 3)
    y = forward(P, x).permute(0, 2, 3, 4, 1).reshape(B, Lx * Ly * Lz, 16)
    m = torch.as_tensor(np.asarray(mask, dtype=np.float64))
    t = torch.as_tensor(np.asarray(target, dtype=np.float64))
    d = (y[:, :, :5] - t) * m[:, :, None]
    loss = (d * d).sum() / m.sum()
    loss.backward()
    return y.detach().numpy(), float(loss.detach()), grads_flat(P)
