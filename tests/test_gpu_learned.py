"""The learned interface-state correction on the GPU, checked against the
float64 oracle (oracle/mlp.py):

* coarsening of a fine snapshot (FP64 kernel): prim / faces / targets equal
  to round-off (relative 1e-12);
* batch assembly (FP32 features rounded to bfloat16): features within one
  bfloat16 rounding plus FP32 error, targets to relative 1e-4;
* BF16 tensor-core forward and gradient: against the oracle evaluated with
  the same bfloat16 rounding of weights and layer inputs, relative L2 error
  below 2e-2 (bfloat16 keeps 8 significant bits);
* the fused learned reconstruction in the solver: PLM states plus the
  network correction within the same tolerance, bit-identical to plain PLM
  when the correction is zero or every stencil is out of the trained range;
* training lowers the loss on held-out snapshots.
"""
import os
import sys

import numpy as np
import pytest

import idefix_gb300 as ig
from idefix_gb300 import ic
from mhd_state import extract

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp  # noqa: E402

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GAMMA = 5.0 / 3.0


@pytest.fixture(scope="module", autouse=True)
def built():
    from idefix_gb300 import build

    build.build_library()
    ig.load_library()


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _fine(n, seed):
    Vc, Vs = ic.turbulence_3d(n, seed=seed, kmax=4)
    return Vc, Vs


def _coarsen_gpu(Vc, Vs, n, r):
    from idefix_gb300 import learned

    dvc = torch.from_numpy(Vc).cuda()
    dvs = torch.from_numpy(Vs).cuda()
    return learned.coarsen(dvc, dvs, n, 2, r, GAMMA)


def _oracle_coarse(Vc, Vs, n, r):
    vc, vs = extract(3, (n, n, n), 2, Vc, Vs)
    faces = [vs[0][:, :, :n], vs[1][:, :n, :], vs[2][:n, :, :]]
    prim, cf = mlp.downsample(vc, faces, r, GAMMA)
    return prim, cf, mlp.face_layers(vc, r)


def test_coarsen_matches_oracle():
    n, r = 32, 4
    Vc, Vs = _fine(n, 11)
    prim, faces, tg = _coarsen_gpu(Vc, Vs, n, r)
    p0, f0, t0 = _oracle_coarse(Vc, Vs, n, r)
    assert _rel(prim.cpu().numpy(), p0) < 1e-12
    assert _rel(faces.cpu().numpy(), f0) < 1e-12
    assert _rel(tg.cpu().numpy(), t0) < 1e-12


def _mix64(z):
    M = (1 << 64) - 1
    z = (z + 0x9E3779B97F4A7C15) & M
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    return z ^ (z >> 31)


def _dataset(seeds, n=32, r=4):
    prims, tgts = [], []
    for s in seeds:
        prim, _, tg = _coarsen_gpu(*_fine(n, s), n, r)
        prims.append(prim.float())
        tgts.append(tg.float())
    return torch.stack(prims).contiguous(), torch.stack(tgts).contiguous()


def test_batch_assembly_matches_oracle():
    from idefix_gb300 import learned

    prims, tgts = _dataset([21, 22])
    tr = learned.Trainer(max_batch=256)
    tr.set_dataset(prims, tgts, GAMMA)
    B, seed, base = 200, 77, 1000
    X, T = tr.batch(B, seed, base)
    X = X.float().cpu().numpy()
    T = T.cpu().numpy()
    P = prims.double().cpu().numpy()
    TG = tgts.double().cpu().numpy()
    nc = P.shape[2]
    ncell = nc**3
    feats = {}
    for i in range(B):
        h = _mix64(seed ^ _mix64(base + i))
        snap, cell, d = h % 2, (h >> 16) % ncell, (h >> 48) % 3
        key = (snap, d)
        if key not in feats:
            feats[key] = (mlp.features(P[snap], d, GAMMA), mlp.targets(P[snap], TG[snap], d, GAMMA))
        fx, ft = feats[key]
        assert np.allclose(X[i, :216], fx[cell], rtol=1e-2, atol=2e-3), i
        assert np.all(X[i, 216:] == 0)
        scale = max(1.0, np.max(np.abs(ft[cell])))
        assert np.max(np.abs(T[i] - ft[cell])) < 1e-4 * scale, i


def test_forward_and_gradient_match_oracle():
    from idefix_gb300 import learned

    rng = np.random.default_rng(5)
    params = mlp.init_params(3, out_scale=0.5)
    B = 384
    Xf = rng.standard_normal((B, 216)) * 0.3
    Tn = rng.standard_normal((B, 16)) * 0.1
    Xb = torch.zeros((B, 224), dtype=torch.float32)
    Xb[:, :216] = torch.from_numpy(Xf).float()
    Xb = Xb.to(torch.bfloat16).cuda()
    Td = torch.from_numpy(Tn).float().cuda()
    tr = learned.Trainer(max_batch=512, params=params.astype(np.float32))
    Xq = Xb.float().cpu().numpy()[:, :216].astype(np.float64)
    p32 = params.astype(np.float32).astype(np.float64)
    Y = tr.forward(Xb).cpu().numpy()
    Y0, _ = mlp.forward(p32, Xq, quant=True)
    assert _rel(Y, Y0) < 2e-2
    g, loss = tr.grad(Xb, Td)
    l0, g0 = mlp.loss_and_grad(p32, Xq, Tn.astype(np.float32).astype(np.float64), quant=True)
    assert abs(loss - l0) < 2e-2 * l0
    G, G0 = mlp.unpack(g), mlp.unpack(g0)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
        assert _rel(G[k], G0[k]) < 2e-2, k


def _learned_block(n, params, fmin=None, fmax=None, order="learned"):
    blk = ig.GpuBlock(3, (n, n, n), order=order, cfl=0.6, first_dt=1e-4)
    if order == "learned":
        blk.set_learned(params, fmin, fmax)
    return blk


def test_fused_reconstruction_matches_oracle():
    n = 16
    Vc, Vs = _fine(n, 31)
    params = mlp.init_params(4, out_scale=0.2).astype(np.float32)
    blk = _learned_block(n, params)
    blk.upload(Vc, Vs)
    ls = blk.learned_states()
    vc, _ = extract(3, (n, n, n), 2, *blk.download())
    p64 = params.astype(np.float64)
    g = 2
    a = slice(g, g + n)
    for d in range(3):
        X = mlp.features(vc, d, GAMMA)
        Y, _ = mlp.forward(p64, X, quant=True)
        vm, vp = mlp.plm_states(vc, d)
        sc = mlp.var_scale(mlp._rotate_vars(vc, d), GAMMA).reshape(8, -1)
        r = mlp.rot(d)
        solver_var = [0, 1 + r[0], 1 + r[1], 1 + r[2], 4, 5 + r[0], 5 + r[1], 5 + r[2]]
        cm = vm + Y[:, 0:8].T * sc
        cp = vp + Y[:, 8:16].T * sc
        # cells whose corrected density or pressure is not positive keep PLM
        fall = (cm[0] <= 0) | (cm[4] <= 0) | (cp[0] <= 0) | (cp[4] <= 0)
        for face, plm in ((0, vm), (1, vp)):
            corr = np.where(fall[None, :], plm, plm + Y[:, face * 8:face * 8 + 8].T * sc)
            for rv in range(8):
                if rv == 5:
                    continue
                got = ls[d, face * 8 + solver_var[rv]][a, a, a].ravel()
                want = corr[rv]
                dev = np.max(np.abs(got - want)) / np.max(np.abs(corr[rv] - plm[rv]) + 1e-300)
                assert dev < 5e-2, (d, face, rv, dev)
    blk.close()


def test_zero_correction_and_full_fallback_are_plain_plm():
    n = 16
    Vc, Vs = _fine(n, 41)
    plain = ig.GpuBlock(3, (n, n, n), order="plm", cfl=0.6, first_dt=1e-4)
    plain.upload(Vc, Vs)
    plain.run(max_cycles=4)
    ref = plain.download()
    zero = mlp.init_params(5, out_scale=0.0).astype(np.float32)  # W3 = b3 = 0
    blk = _learned_block(n, zero)
    blk.upload(Vc, Vs)
    blk.run(max_cycles=4)
    out = blk.download()
    assert np.array_equal(out[0], ref[0]) and np.array_equal(out[1], ref[1])
    cells, fall = blk.learned_stats()
    assert cells > 0 and fall == 0
    # an empty trained range: every cell falls back
    big = mlp.init_params(6, out_scale=1.0).astype(np.float32)
    lo = np.ones(216, dtype=np.float32)
    hi = -np.ones(216, dtype=np.float32)
    blk2 = _learned_block(n, big, lo, hi)
    blk2.upload(Vc, Vs)
    blk2.run(max_cycles=4)
    out2 = blk2.download()
    assert np.array_equal(out2[0], ref[0]) and np.array_equal(out2[1], ref[1])
    cells2, fall2 = blk2.learned_stats()
    assert cells2 == fall2 > 0


def test_learned_run_keeps_div_b_and_conservation():
    n = 16
    Vc, Vs = _fine(n, 51)
    params = mlp.init_params(7, out_scale=0.05).astype(np.float32)
    blk = _learned_block(n, params)
    blk.upload(Vc, Vs)
    blk.set_boundaries()
    blk.prim_to_cons()
    u0 = blk.download_cons()
    blk.run(max_cycles=6)
    assert blk.check_divb() < 1e-11
    u1 = blk.download_cons()
    a = slice(2, 2 + n)
    for v in (0, 1, 2, 3, 4):
        s0, s1 = u0[v][a, a, a].sum(), u1[v][a, a, a].sum()
        assert abs(s1 - s0) <= 1e-11 * max(1.0, abs(u0[0][a, a, a].sum())), v


def test_training_lowers_held_out_loss():
    from idefix_gb300 import learned

    train_p, train_t = _dataset([61, 62, 63], n=64)
    hold_p, hold_t = _dataset([64], n=64)
    tr = learned.Trainer(max_batch=2048)
    tr.set_dataset(train_p, train_t, GAMMA)
    losses = tr.train(300, 2048, lr=2e-3, lr_end=1e-4, seed=1)
    assert np.all(np.isfinite(losses))
    assert losses[-20:].mean() < losses[:5].mean()
    tr.set_dataset(hold_p, hold_t, GAMMA)
    loss, loss_zero = tr.eval(2048, seed=99)
    assert loss < 0.8 * loss_zero, (loss, loss_zero)
