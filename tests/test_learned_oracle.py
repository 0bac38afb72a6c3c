"""CPU checks of the learned-correction oracle (oracle/mlp.py), which the GPU
tests use as the oracle of the tensor-core kernels: its gradient against
central finite differences and, with its Adam step, against torch's
autograd and optimiser; its coarsening against the conservation laws
and div B = 0, and its features / PLM states on states with known answers.
"""
import os
import sys

import numpy as np
import pytest

from idefix_gb300 import ic
from mhd_state import extract

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp  # noqa: E402


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = mlp.init_params(1, out_scale=0.5)
    X = rng.standard_normal((7, mlp.NIN)) * 0.5
    T = rng.standard_normal((7, mlp.NOUT))
    _, g = mlp.loss_and_grad(p, X, T)
    eps = 1e-6
    for i in rng.choice(mlp.NPARAM, 40, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (mlp.loss_and_grad(pp, X, T)[0] - mlp.loss_and_grad(pm, X, T)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), i


def test_masked_outputs_have_no_gradient():
    rng = np.random.default_rng(4)
    p = mlp.init_params(2, out_scale=0.5)
    X = rng.standard_normal((5, mlp.NIN))
    T = rng.standard_normal((5, mlp.NOUT))
    _, g = mlp.loss_and_grad(p, X, T)
    W3 = mlp.unpack(g)["W3"]
    b3 = mlp.unpack(g)["b3"]
    assert np.all(W3[:, [5, 13]] == 0) and np.all(b3[[5, 13]] == 0)


def _fine_compact(n=16, seed=5):
    Vc, Vs = ic.turbulence_3d(n, seed=seed, kmax=3)
    vc, vs = extract(3, (n, n, n), 2, Vc, Vs)
    faces = [vs[0][:, :, :n], vs[1][:, :n, :], vs[2][:n, :, :]]
    return vc, faces


def test_coarsening_conserves_and_keeps_div_b_zero():
    gamma = 5.0 / 3.0
    vc, faces = _fine_compact()
    prim, cf = mlp.downsample(vc, faces, 4, gamma)
    rho, v, p, B = vc[0], vc[1:4], vc[4], vc[5:8]
    E = p / (gamma - 1) + 0.5 * rho * (v * v).sum(0) + 0.5 * (B * B).sum(0)
    crho, cv, cp, cB = prim[0], prim[1:4], prim[4], prim[5:8]
    cE = cp / (gamma - 1) + 0.5 * crho * (cv * cv).sum(0) + 0.5 * (cB * cB).sum(0)
    r3 = 64.0
    assert abs(crho.sum() * r3 - rho.sum()) <= 1e-12 * rho.sum()
    for k in range(3):
        assert abs((crho * cv[k]).sum() * r3 - (rho * v[k]).sum()) <= 1e-12 * rho.sum()
    assert abs(cE.sum() * r3 - E.sum()) <= 1e-12 * E.sum()
    # coarse div B from the coarse faces (periodic)
    div = sum(np.roll(cf[d], -1, axis=2 - d) - cf[d] for d in range(3))
    assert np.max(np.abs(div)) < 1e-12
    fine_div = sum(np.roll(faces[d], -1, axis=2 - d) - faces[d] for d in range(3))
    assert np.max(np.abs(fine_div)) < 1e-12


def test_features_and_plm_known_answers():
    gamma = 1.4
    n = 6
    prim = np.zeros((8, n, n, n))
    prim[0], prim[4] = 2.0, 3.0
    prim[1:4] = np.array([0.3, -0.2, 0.1])[:, None, None, None]
    prim[5:8] = np.array([0.5, 0.25, -1.0])[:, None, None, None]
    for d in range(3):
        X = mlp.features(prim, d, gamma)
        cs = np.sqrt(gamma * 3.0 / 2.0)
        sb = np.sqrt(2.0) * cs
        r = mlp.rot(d)
        B = prim[5:8, 0, 0, 0][r]
        expect = np.zeros(mlp.NIN)
        for k in range(3):
            expect[(5 + k) * 27:(6 + k) * 27] = B[k] / sb
        assert np.allclose(X, expect[None, :], rtol=0, atol=1e-15)
    # PLM of a linear profile along x: the van Leer slope is exact
    lin = np.zeros((8, n, n, n))
    lin[:] = 1.0
    lin[0] = 1.0 + 0.1 * np.arange(n)[None, None, :]
    vm, vp = mlp.plm_states(lin, 0)
    inner = vm[0].reshape(n, n, n)[:, :, 1:-1]
    assert np.allclose(inner, (1.0 + 0.1 * np.arange(1, n - 1) - 0.05)[None, None, :])
    assert np.allclose(vp[0].reshape(n, n, n)[:, :, 1:-1], (1.0 + 0.1 * np.arange(1, n - 1) + 0.05)[None, None, :])


def test_face_targets_are_exact_for_linear_profiles():
    # a field linear in x: the extrapolation from the two fine layers next
    # to a coarse face gives the field's value on that face
    r, nc = 4, 3
    nf = nc * r
    x = (np.arange(nf) + 0.5) / nf
    fine = np.ones((8, nf, nf, nf))
    fine[0] = 2.0 + 3.0 * x[None, None, :]
    t = mlp.face_layers(fine, r)
    faces = np.arange(nc + 1) / nc
    got_left = t[0, 0].reshape(nc, nc, nc)[0, 0, :]
    got_right = t[0, 8].reshape(nc, nc, nc)[0, 0, :]
    assert np.allclose(got_left, 2.0 + 3.0 * faces[:-1])
    assert np.allclose(got_right, 2.0 + 3.0 * faces[1:])
    # r = 1: the cell values themselves
    t1 = mlp.face_layers(fine[:, :3, :3, :3], 1)
    assert np.allclose(t1[0, 0], fine[0, :3, :3, :3].ravel())


def test_gradient_and_adam_match_torch_autograd():
    """the oracle's hand-written backward pass and Adam step against torch's
    autograd and torch.optim.Adam, float64 on the CPU"""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(6)
    p = mlp.init_params(3, out_scale=0.5)
    X = rng.standard_normal((9, mlp.NIN)) * 0.5
    T = rng.standard_normal((9, mlp.NOUT))
    P = {k: torch.tensor(v.copy(), dtype=torch.float64, requires_grad=True) for k, v in mlp.unpack(p).items()}
    names = ("W1", "b1", "W2", "b2", "W3", "b3")
    opt = torch.optim.Adam([P[k] for k in names], lr=1e-3, betas=(0.9, 0.999), eps=1e-8)
    Xt, Tt = torch.tensor(X), torch.tensor(T)
    mask = torch.tensor(mlp.LOSS_MASK)
    m = np.zeros(mlp.NPARAM)
    v = np.zeros(mlp.NPARAM)
    for step in range(1, 4):
        opt.zero_grad()
        H1 = torch.nn.functional.silu(Xt @ P["W1"] + P["b1"])
        H2 = torch.nn.functional.silu(H1 @ P["W2"] + P["b2"])
        Y = H2 @ P["W3"] + P["b3"]
        loss = (((Y - Tt) * mask) ** 2).sum() / X.shape[0]
        loss.backward()
        ref_g = np.concatenate([P[k].grad.detach().numpy().ravel() for k in names])
        ours_loss, g = mlp.loss_and_grad(p, X, T)
        assert abs(ours_loss - loss.item()) <= 1e-12 * abs(loss.item())
        assert np.max(np.abs(g - ref_g)) <= 1e-12 * max(1.0, np.max(np.abs(ref_g)))
        opt.step()
        p, m, v = mlp.adam(p, g, m, v, step, 1e-3)
        ref_p = np.concatenate([P[k].detach().numpy().ravel() for k in names])
        assert np.max(np.abs(p - ref_p)) <= 1e-12
