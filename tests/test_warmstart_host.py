"""Host-side pieces of the learned warm start that need no GPU: the lattice
symmetries used to augment training samples leave the oracle's Landau-de
Gennes energy (L1-L3, homeotropic walls and sphere) unchanged, and the c4
generator draws its geometry from the documented ranges."""
import importlib

import numpy as np
import pytest
import torch


def _sym(oracle, sol, Q, types):
    s = oracle.System(sol["L"], Ls=(*sol["Ls"], 0.0))
    s.random_nematic(0)
    s.types[:] = 0
    for kind, W, S0 in sol["objects"]:
        s.objs[s.nobj].kind, s.objs[s.nobj].W, s.objs[s.nobj].S0 = kind, W, S0
        s.nobj += 1
    s.Q[:] = Q
    s.types[:] = types
    return s


@pytest.mark.parametrize("flips,swap", [((1, 0, 0), False), ((0, 1, 0), False), ((0, 0, 1), False),
                                        ((0, 0, 0), True), ((1, 1, 1), True), ((1, 0, 1), True)])
def test_augmentation_preserves_energy(qmin, oracle, flips, swap):
    w = importlib.import_module("qmin_gb300.workloads")
    ws = importlib.import_module("qmin_gb300.warmstart")
    sol = w.c4_solve(7, side=16)
    L = sol["L"]
    n = L[0] * L[1] * L[2]
    t5 = torch.as_tensor(sol["Q"])
    x16 = torch.zeros((n, 16), dtype=torch.float64)
    x16[:, :5] = t5
    x16[:, 5] = torch.as_tensor(sol["types"]).double()
    t2, x2 = ws._augment(t5, x16, L, flips, swap)
    types2 = x2[:, 5].round().to(torch.int64).numpy().astype(np.int32)
    assert np.array_equal(x2[:, :5].numpy(), t2.numpy())
    e0 = _sym(oracle, sol, sol["Q"], sol["types"]).energy()
    e1 = _sym(oracle, sol, t2.numpy(), types2).energy()
    assert abs(e1[0] - e0[0]) <= 1e-12 * abs(e0[0]), (e0[0], e1[0])


def test_c4_generator_ranges(qmin):
    w = importlib.import_module("qmin_gb300.workloads")
    for seed in range(20):
        s = w.c4_solve(seed)
        (cx, cy, cz), r, W = s["sphere"]
        assert 6.4 <= r <= 12.8 and 1.0 <= W <= 10.0
        assert 0 <= cx < 64 and 0 <= cy < 64 and r + 3 <= cz <= 60 - r
        assert len(s["objects"]) == 3
        assert (s["types"].reshape(64, 64, 64)[0] == 1).all() and (s["types"].reshape(64, 64, 64)[63] == 2).all()
    a = w.c4_solve(3)
    b = w.c4_solve(3, qseed=99)
    assert np.array_equal(a["types"], b["types"]) and not np.array_equal(a["Q"], b["Q"])


def test_crop_origins(qmin):
    """Crops of the patch-tiled fine-tuning: a 64-site pitch with the last crop
    flush with the far face, so that every site of the axis is covered."""
    import importlib
    ws = importlib.import_module("qmin_gb300.warmstart")
    assert ws.crop_origins(200, 64) == [0, 64, 128, 136]
    assert ws.crop_origins(400, 64) == [0, 64, 128, 192, 256, 320, 336]
    assert ws.crop_origins(128, 64) == [0, 64]
    assert ws.crop_origins(64, 64) == [0]
    for n in (64, 100, 200, 333, 400):
        o = ws.crop_origins(n, 64)
        covered = set()
        for a in o:
            covered.update(range(a, a + 64))
        assert covered == set(range(n))
    with pytest.raises(ValueError):
        ws.crop_origins(48, 64)
