"""Learned warm start: dataset generation with the batched FIRE path, training
of the warm-start net on the GPU, and the FIRE-finishes-and-judges protocol.

Protocol: a warm-started solve starts from the net's prediction (object sites
keep their imposed Q), FIRE in FP32 finishes it to forceMax < cutoff, and it
counts only if the final state's forceMax, recomputed in FP64, is below the
cutoff and its FP64 energy is within `energy_tol` (relative) of the energy the
plain FP64 FIRE reaches from the same initial field; otherwise the solve is
restarted from the plain initial field in FP32 and the restart's time is
charged to the warm-started run.

PyTorch serves here as host glue only: device storage of the dataset, index
shuffling and copies into the net's input buffers.  All network arithmetic
runs in the native library (qmin_warmnet_*)."""
import math
import time

import numpy as np

from . import FP32, FP64, Batch, Lattice, WarmNet, warmnet_init_params


def _torch():
    import torch
    return torch


def set_up_lattice(sol, precision, Q=None):
    lat = Lattice(sol["L"], precision)
    a, b, c = sol["consts"]
    lat.set_params(a, b, c, *sol["Ls"], E=sol.get("E"), H=sol.get("H"))
    lat.set_objects(sol["objects"])
    lat.set_state(sol["Q"] if Q is None else Q, sol["types"])
    return lat


def fp64_check(sol, Q):
    """(forceMax, E / NActive) of the state Q evaluated in FP64:
    forceMax = sqrt(sum_i F_i ._QT F_i) / nTotal (energyMinimizerFIRE.cpp:110)."""
    lat = set_up_lattice(sol, FP64, Q)
    F = lat.force()
    dot = (F * F).sum(axis=1) + F[:, 0] * F[:, 3]
    fm = math.sqrt(max(float(dot.sum()), 0.0)) / lat.n_active()
    e = lat.energy()[0]
    lat.close()
    return fm, e


def solve_batch(sols, precision, Qs=None, force_cutoff=1e-6, max_iterations=30000):
    """FIRE (CLI parameters) on every solve together; returns the per-solve
    iteration counts and forceMax, the final Q (host AoS) and the seconds the
    minimisation took (device work synchronised)."""
    b = Batch([s["L"] for s in sols], precision)
    a, bb, c = sols[0]["consts"]
    b.set_params(a, bb, c, *sols[0]["Ls"])
    for k, s in enumerate(sols):
        b.set_solve(k, s["Q"] if Qs is None else Qs[k], s["types"], s["objects"])
    b.fire_init(force_cutoff=force_cutoff)
    t0 = time.perf_counter()
    r = b.fire_run(max_iterations)
    sec = time.perf_counter() - t0
    Q = [b.get_solve(k) for k in range(len(sols))]
    b.close()
    return dict(iterations=r["iterations"], forceMax=r["forceMax"], converged=r["converged"], Q=Q, seconds=sec)


class FeatureNet:
    """A batch-1 inference net used to turn a lattice's initial state into input features."""

    def __init__(self, L):
        self.net = WarmNet(1, L, train=False)
        self.x, self.y, self.m = self.net.torch_views()

    def features(self, sol):
        torch = _torch()
        q = torch.as_tensor(np.ascontiguousarray(sol["Q"].T)).cuda()
        t = torch.as_tensor(sol["types"].astype(np.int8)).cuda()
        torch.cuda.synchronize()
        self.net.features(0, q.data_ptr(), FP64, q.shape[1], t.data_ptr(), sol["objects"])
        self.net.sync()
        return self.x[0].clone(), self.m[0].clone()


def make_dataset(make_solve, seeds, group=256, log=print):
    """Features, FIRE targets (FP32, forceMax < 1e-6) and masks of every seed,
    resident on the device: x bf16 [n, sites, 16], target f32 [n, sites, 5],
    mask u8 [n, sites]."""
    torch = _torch()
    first = make_solve(seeds[0])
    L = first["L"]
    n, sites = len(seeds), L[0] * L[1] * L[2]
    X = torch.empty((n, sites, 16), dtype=torch.bfloat16, device="cuda")
    T = torch.empty((n, sites, 5), dtype=torch.float32, device="cuda")
    M = torch.empty((n, sites), dtype=torch.uint8, device="cuda")
    fn = FeatureNet(L)
    its = []
    t0 = time.perf_counter()
    for g0 in range(0, n, group):
        sols = [first if (g0 + k == 0) else make_solve(seeds[g0 + k]) for k in range(min(group, n - g0))]
        r = solve_batch(sols, FP32)
        its.extend(int(i) for i in r["iterations"])
        for k, s in enumerate(sols):
            X[g0 + k], M[g0 + k] = fn.features(s)
            T[g0 + k] = torch.as_tensor(r["Q"][k].astype(np.float32)).cuda()
        log(f"dataset {g0 + len(sols)}/{n}: FIRE {r['seconds']:.1f} s, converged {r['converged']}/{len(sols)}, "
            f"median iterations {int(np.median(r['iterations']))}, elapsed {time.perf_counter() - t0:.0f} s")
    fn.net.close()
    return dict(x=X, target=T, mask=M, iterations=np.array(its), L=L)


def fire_lattice(sol, precision=FP32, force_cutoff=1e-6, max_iterations=30000):
    """Plain FIRE (CLI parameters, dt 5e-4) on one lattice through the
    single-lattice path; returns (final Q host AoS, iterations, seconds)."""
    lat = set_up_lattice(sol, precision)
    lat.fire_init(dt=5e-4, force_cutoff=force_cutoff)
    t0 = time.perf_counter()
    r = lat.fire_run(max_iterations)
    sec = time.perf_counter() - t0
    Q = lat.get_state()[0]
    lat.close()
    return Q, int(r["iterations"]), sec


def crop_origins(n, side):
    """Origins of side-long crops along an axis of n sites: a pitch of `side`,
    the last crop flush with the far face (it overlaps its neighbour when
    side does not divide n)."""
    if n < side:
        raise ValueError(f"an axis of {n} sites holds no crop of {side}")
    o = list(range(0, n - side + 1, side))
    if o[-1] != n - side:
        o.append(n - side)
    return o


def make_crop_dataset(lattices, side=64, border=8, log=print):
    """Patch-tiled samples of large lattices: each lattice is minimised whole
    (FP32 FIRE to forceMax < 1e-6), its features are computed whole, and
    side^3 crops at origins spaced by `side` (the last one flush with the far
    face) become samples: features, final Q and the moved-site mask with a
    `border`-site band at every crop face taken out (the net sees zeros past a
    crop's faces, where the lattice had context).  Same layout as make_dataset."""
    torch = _torch()
    crops = []
    for sol in lattices:
        L = sol["L"]
        Q, its, sec = fire_lattice(sol)
        fn = FeatureNet(L)
        x, m = fn.features(sol)
        fn.net.close()
        x3 = x.view(L[2], L[1], L[0], 16)
        m3 = m.view(L[2], L[1], L[0])
        t3 = torch.as_tensor(Q.astype(np.float32)).cuda().view(L[2], L[1], L[0], 5)

        for z0 in crop_origins(L[2], side):
            for y0 in crop_origins(L[1], side):
                for x0 in crop_origins(L[0], side):
                    sl = (slice(z0, z0 + side), slice(y0, y0 + side), slice(x0, x0 + side))
                    mm = m3[sl].clone()
                    mm[:border], mm[-border:] = 0, 0
                    mm[:, :border], mm[:, -border:] = 0, 0
                    mm[:, :, :border], mm[:, :, -border:] = 0, 0
                    crops.append((x3[sl].reshape(-1, 16).clone(), t3[sl].reshape(-1, 5).clone(), mm.reshape(-1)))
        log(f"crops: lattice {L} FIRE {its} iterations in {sec:.2f} s, {len(crops)} crops so far")
        del x3, m3, t3, x, m
    n = len(crops)
    sites = side ** 3
    X = torch.empty((n, sites, 16), dtype=torch.bfloat16, device="cuda")
    T = torch.empty((n, sites, 5), dtype=torch.float32, device="cuda")
    M = torch.empty((n, sites), dtype=torch.uint8, device="cuda")
    for k, (x, t, m) in enumerate(crops):
        X[k], T[k], M[k] = x, t, m
    return dict(x=X, target=T, mask=M, iterations=np.zeros(0), L=(side, side, side))


def concat_datasets(parts):
    """One dataset from several with the same sample shape."""
    torch = _torch()
    assert len({tuple(p["L"]) for p in parts}) == 1
    return dict(x=torch.cat([p["x"] for p in parts]), target=torch.cat([p["target"] for p in parts]),
                mask=torch.cat([p["mask"] for p in parts]),
                iterations=np.concatenate([np.asarray(p["iterations"]) for p in parts]), L=parts[0]["L"])


# Lattice symmetries used for augmentation.  Q = (Qxx, Qxy, Qxz, Qyy, Qyz):
# the mirror x -> -x negates Qxy and Qxz, y -> -y negates Qxy and Qyz,
# z -> -z negates Qxz and Qyz; swapping x and y exchanges Qxx<->Qyy and Qxz<->Qyz.
# The bulk, L1-L3 and anchoring terms are invariant under all of them (the
# chiral L4 term is not: augmentation is for L4 = 0 data only).
_MIRROR_SIGN = {0: (1, -1, -1, 1, 1), 1: (1, -1, 1, 1, -1), 2: (1, 1, -1, 1, -1)}  # axis x, y, z
_SWAP_XY = (3, 1, 4, 0, 2)


def _augment(t5, x16, L, flips, swap):
    """Apply mirrors (flips[a] for axis a = x, y, z) and an x<->y swap to one
    sample's target [sites, 5] and features [sites, 16] (torch, device)."""
    torch = _torch()
    Lx, Ly, Lz = L
    t = t5.view(Lz, Ly, Lx, 5)
    x = x16.view(Lz, Ly, Lx, 16)
    dims = [2 - a for a in range(3) if flips[a]]  # array dims: z = 0, y = 1, x = 2
    sign = torch.ones(5, device=t5.device)
    for a in range(3):
        if flips[a]:
            sign = sign * torch.tensor(_MIRROR_SIGN[a], device=t5.device, dtype=sign.dtype)
    if dims:
        # mirrors first (flip the sites, then the odd components)...
        t = torch.flip(t, dims) * sign
        x = torch.flip(x, dims)
        x = torch.cat([x[..., :5] * sign.to(x.dtype), x[..., 5:]], dim=-1)  # +-1: exact in any dtype
    if swap:
        # ...then the x<->y swap of sites and components
        t = t.transpose(1, 2)[..., list(_SWAP_XY)]
        xq = x[..., :5][..., list(_SWAP_XY)]
        x = torch.cat([xq, x[..., 5:]], dim=-1).transpose(1, 2)
    return t.reshape(-1, 5), x.reshape(-1, 16)


def train(data, epochs=10, batch=8, lr=1e-3, lr_min=2e-5, seed=0, params=None, augment=True, log=print,
          log_every=100):
    """Adam on the masked MSE; cosine learning-rate decay; each sample drawn
    under a random lattice symmetry (mirrors, x<->y swap on square x-y
    cross-sections) when `augment`; returns (params, per-epoch mean losses)."""
    torch = _torch()
    L, n = data["L"], data["x"].shape[0]
    net = WarmNet(batch, L, train=True)
    net.set_stream(torch.cuda.current_stream().cuda_stream)
    net.set_params(warmnet_init_params(seed) if params is None else params)
    xv, _yv, mv = net.torch_views()
    gen = torch.Generator(device="cpu")
    gen.manual_seed(seed)
    steps_per_epoch = n // batch
    total = epochs * steps_per_epoch
    hist, step = [], 0
    t0 = time.perf_counter()
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen)
        losses = []
        for s in range(steps_per_epoch):
            idx = perm[s * batch:(s + 1) * batch].cuda()
            xb = data["x"].index_select(0, idx)
            mb = data["mask"].index_select(0, idx)
            tgt = data["target"].index_select(0, idx).contiguous()
            if augment:
                draws = torch.randint(0, 2, (batch, 4), generator=gen).tolist()
                for k in range(batch):
                    fl, sw = draws[k][:3], bool(draws[k][3]) and L[0] == L[1]
                    if any(fl) or sw:
                        tgt[k], xb[k] = _augment(tgt[k], xb[k], L, fl, sw)
                        m3 = mb[k].view(L[2], L[1], L[0])
                        dims = [2 - a for a in range(3) if fl[a]]
                        if dims:
                            m3 = torch.flip(m3, dims)
                        if sw:
                            m3 = m3.transpose(1, 2)
                        mb[k] = m3.reshape(-1)
            xv.copy_(xb)
            mv.copy_(mb)
            net.forward()
            want = (s % log_every == 0) or s == steps_per_epoch - 1
            loss = net.backward(tgt.data_ptr(), want_loss=want)
            if want:
                losses.append(loss)
            lr_t = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * step / max(total, 1)))
            net.adam_step(lr_t)
            step += 1
        torch.cuda.synchronize()
        hist.append(float(np.mean(losses)))
        log(f"epoch {ep + 1}/{epochs}: loss {hist[-1]:.3e}, lr {lr_t:.2e}, elapsed {time.perf_counter() - t0:.0f} s")
    p = net.get_params()
    net.close()
    return p, hist


def predict(params, sols, batch=8):
    """The net's predicted Q for every solve (host AoS, object sites from Q0),
    and the seconds the inference took."""
    torch = _torch()
    L = sols[0]["L"]
    net = WarmNet(batch, L, train=False)
    net.set_params(params)
    _x, yv, _m = net.torch_views()
    out, sec = [], 0.0
    for g0 in range(0, len(sols), batch):
        grp = sols[g0:g0 + batch]
        keep = []
        for k, s in enumerate(grp):
            q = torch.as_tensor(np.ascontiguousarray(s["Q"].T)).cuda()
            t = torch.as_tensor(s["types"].astype(np.int8)).cuda()
            keep.append((q, t))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k, s in enumerate(grp):
            q, t = keep[k]
            net.features(k, q.data_ptr(), FP64, q.shape[1], t.data_ptr(), s["objects"])
        net.forward()
        net.sync()
        sec += time.perf_counter() - t0
        y = yv[:len(grp), :, :5].cpu().numpy().astype(np.float64)
        for k, s in enumerate(grp):
            Q = y[k].copy()
            obj = s["types"] > 0
            Q[obj] = s["Q"][obj]
            out.append(Q)
    net.close()
    return out, sec


def evaluate(params, sols, force_cutoff=1e-6, energy_tol=1e-4, plain=None, log=print):
    """The protocol over `sols`: plain FP64 FIRE, warm start + FP32 FIRE,
    FP64 judgement, FP32 restarts of the solves that fail."""
    if plain is None:
        plain = solve_batch(sols, FP64, force_cutoff=force_cutoff)
        plain["E"] = np.array([fp64_check(s, q)[1] for s, q in zip(sols, plain["Q"])])
    Qw, t_inf = predict(params, sols)
    warm = solve_batch(sols, FP32, Qs=Qw, force_cutoff=force_cutoff)
    fm64, E64 = zip(*[fp64_check(s, q) for s, q in zip(sols, warm["Q"])])
    fm64, E64 = np.array(fm64), np.array(E64)
    rel = np.abs(E64 - plain["E"]) / np.abs(plain["E"])
    ok = (fm64 < force_cutoff) & (rel <= energy_tol) & (warm["iterations"] < 30000)
    fail = [k for k in range(len(sols)) if not ok[k]]
    t_restart, its_restart = 0.0, np.zeros(0, dtype=np.int64)
    if fail:
        rr = solve_batch([sols[k] for k in fail], FP32, force_cutoff=force_cutoff)
        t_restart, its_restart = rr["seconds"], rr["iterations"]
    plain32 = solve_batch(sols, FP32, force_cutoff=force_cutoff)
    res = dict(n=len(sols), passed=int(ok.sum()), failed=fail,
               plain_fp64_seconds=plain["seconds"], plain_fp32_seconds=plain32["seconds"],
               warm_inference_seconds=t_inf, warm_fire_seconds=warm["seconds"], restart_seconds=t_restart,
               warm_total_seconds=t_inf + warm["seconds"] + t_restart,
               iterations_plain_fp64=float(np.mean(plain["iterations"])),
               iterations_plain_fp32=float(np.mean(plain32["iterations"])),
               iterations_warm=float(np.mean(warm["iterations"])),
               energy_rel_max=float(rel.max()), energy_rel_median=float(np.median(rel)),
               forcemax64_max=float(fm64.max()),
               failed_detail=[dict(solve=int(k), E_rel_signed=float((E64[k] - plain["E"][k]) / abs(plain["E"][k])),
                                   forceMax_fp64=float(fm64[k]), iterations=int(warm["iterations"][k]))
                              for k in fail])
    log(res)
    return res
