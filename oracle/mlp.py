"""NumPy restatement of the learned interface-state correction — TEST
INFRASTRUCTURE ONLY (imported by tests/ as the oracle of the CUDA kernels;
the product library never imports it).

The reference has no learned component; this file is the mathematical
definition that the CUDA kernels of idefix_gb300/csrc/learned.cu implement,
in float64:

* stencil features: the 3x3x3 primitive stencil (RHO, VX1..3, PRS, BX1..3)
  around a cell, in the frame rotated so that the sweep direction is the
  first axis (cyclic permutation of axes and vector components), scaled by
  the centre cell:  rho/rho_c - 1, (v - v_c)/c_s, p/p_c - 1, B/(sqrt(rho_c) c_s)
  with c_s = sqrt(gamma p_c / rho_c); feature index = var * 27 + cell,
  cell = (dz+1)*9 + (dy+1)*3 + (dx+1) in the rotated frame;
* MLP 216 -> 128 -> 128 -> 16, SiLU, outputs = normalised corrections of
  the cell's minus-face and plus-face states (8 + 8, rotated frame), scaled
  back with the same factors;
* training target: the fine-grid primitives extrapolated to each coarse
  face from the two fine layers next to it (1.5 x outer - 0.5 x next),
  averaged over the face, minus the coarse PLM (van Leer) state;
  the normal field component (taken from the face field by the solver) is
  masked out of the loss;
* coarse state of a fine snapshot: conserved variables averaged over the
  r^3 fine cells, face fields averaged over the r^2 fine faces, cell field =
  mean of the two faces, then ConsToPrim.
"""
import numpy as np

NVAR = 8
NIN = 216
K1 = 224  # NIN padded to a multiple of 32
NH = 128
NOUT = 16
NPARAM = NIN * NH + NH + NH * NH + NH + NH * NOUT + NOUT
LOSS_MASK = np.ones(NOUT)
LOSS_MASK[[5, 13]] = 0.0  # rotated normal field component of both faces

RHO, VX, PRS, BX = 0, 1, 4, 5


def rot(d):
    """axes of the rotated frame (sweep direction first), cyclic"""
    return [(d + 0) % 3, (d + 1) % 3, (d + 2) % 3]


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    o = 0
    out = {}
    for name, shape in (("W1", (NIN, NH)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)),
                        ("W3", (NH, NOUT)), ("b3", (NOUT,))):
        size = int(np.prod(shape))
        out[name] = p[o:o + size].reshape(shape)
        o += size
    return out


def pack(P):
    return np.concatenate([P[k].ravel() for k in ("W1", "b1", "W2", "b2", "W3", "b3")])


def init_params(seed=0, out_scale=0.0):
    """He-style initialisation; the last layer starts at out_scale x (zero
    by default: an untrained network makes no correction)."""
    rng = np.random.default_rng(seed)
    P = {"W1": rng.standard_normal((NIN, NH)) * np.sqrt(2.0 / NIN), "b1": np.zeros(NH),
         "W2": rng.standard_normal((NH, NH)) * np.sqrt(2.0 / NH), "b2": np.zeros(NH),
         "W3": rng.standard_normal((NH, NOUT)) * np.sqrt(2.0 / NH) * out_scale, "b3": np.zeros(NOUT)}
    return pack(P)


def bf16(x):
    """round to the nearest bfloat16 (ties to even), returned as float64"""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, X, quant=False):
    """X[N, 216] -> (Y[N, 16], cache); quant: round weights and the
    activations fed to each layer to bfloat16, as the tensor-core kernels do"""
    P = unpack(params)
    q = bf16 if quant else (lambda a: np.asarray(a, dtype=np.float64))
    X = q(X)
    Z1 = X @ q(P["W1"]) + P["b1"]
    H1 = q(silu(Z1))
    Z2 = H1 @ q(P["W2"]) + P["b2"]
    H2 = q(silu(Z2))
    Y = H2 @ q(P["W3"]) + P["b3"]
    return Y, (X, Z1, H1, Z2, H2)


def loss_and_grad(params, X, T, quant=False):
    """mean over the batch of the masked squared error, and its gradient
    with respect to the packed parameters"""
    P = unpack(params)
    q = bf16 if quant else (lambda a: np.asarray(a, dtype=np.float64))
    Y, (Xq, Z1, H1, Z2, H2) = forward(params, X, quant)
    N = X.shape[0]
    R = (Y - T) * LOSS_MASK
    loss = float(np.sum(R * R) / N)
    dY = 2.0 * R / N
    g = {}
    g["W3"] = H2.T @ dY
    g["b3"] = dY.sum(0)
    dH2 = dY @ q(P["W3"]).T
    dZ2 = dH2 * dsilu(Z2)
    g["W2"] = H1.T @ dZ2
    g["b2"] = dZ2.sum(0)
    dH1 = dZ2 @ q(P["W2"]).T
    dZ1 = dH1 * dsilu(Z1)
    g["W1"] = Xq.T @ dZ1
    g["b1"] = dZ1.sum(0)
    return loss, pack(g)


def adam(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """one Adam step (step counts from 1); returns new (params, m, v)"""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1**step)
    vh = v / (1 - b2**step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


# ---------------------------------------------------------------------------
# stencils, PLM and targets on a periodic compact grid prim[8, nz, ny, nx]
# ---------------------------------------------------------------------------
def _rolled(prim, d, off):
    """prim shifted so that element [c] holds the value at c + off (rotated
    frame offsets off = (o0, o1, o2) along rot(d))"""
    axes = rot(d)
    out = prim
    for a, o in zip(axes, off):
        if o:
            out = np.roll(out, -o, axis=3 - a)  # array axis of direction a
    return out


def _rotate_vars(stencil_vars, d):
    """variable order in the rotated frame"""
    r = rot(d)
    idx = [RHO, VX + r[0], VX + r[1], VX + r[2], PRS, BX + r[0], BX + r[1], BX + r[2]]
    return stencil_vars[idx]


def scales(prim_c, gamma):
    rho, p = prim_c[RHO], prim_c[PRS]
    cs = np.sqrt(gamma * p / rho)
    return rho, cs, p, np.sqrt(rho) * cs


def var_scale(prim_c, gamma):
    """per rotated variable scale (8, ...)"""
    rho, cs, p, sb = scales(prim_c, gamma)
    return np.stack([rho, cs, cs, cs, p, sb, sb, sb])


def features(prim, d, gamma):
    """prim[8, nz, ny, nx] periodic -> X[ncell, 216] in the rotated frame of
    direction d (cells in C order of the compact grid)"""
    c = _rotate_vars(prim, d)
    rho_c, cs, p_c, sb = scales(c, gamma)
    feats = []
    for var in range(NVAR):
        for o2 in (-1, 0, 1):
            for o1 in (-1, 0, 1):
                for o0 in (-1, 0, 1):
                    s = _rotate_vars(_rolled(prim, d, (o0, o1, o2)), d)[var]
                    if var == RHO:
                        f = s / rho_c - 1.0
                    elif var in (1, 2, 3):
                        f = (s - c[var]) / cs
                    elif var == PRS:
                        f = s / p_c - 1.0
                    else:
                        f = s / sb
                    feats.append(f.ravel())
    return np.stack(feats, axis=1)


def vanleer(dvp, dvm):
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(dvp * dvm > 0.0, 2.0 * dvp * dvm / (dvp + dvm), 0.0)


def plm_states(prim, d):
    """van Leer PLM states of every cell along d, rotated variable order:
    (minus-face [8, ncell], plus-face [8, ncell])"""
    w0 = _rotate_vars(_rolled(prim, d, (-1, 0, 0)), d)
    w1 = _rotate_vars(prim, d)
    w2 = _rotate_vars(_rolled(prim, d, (1, 0, 0)), d)
    dd = vanleer(w2 - w1, w1 - w0)
    return (w1 - 0.5 * dd).reshape(NVAR, -1), (w1 + 0.5 * dd).reshape(NVAR, -1)


def face_layers(fine_prim, r):
    """fine prim[8, nf, nf, nf] -> raw face targets [3, 16, nc^3]: for each
    direction d, the fine primitives extrapolated to the two faces of every
    coarse cell along d from the two fine layers next to each face
    (1.5 x outer - 0.5 x next; the outer layer alone when r = 1), averaged
    over the face (rotated variable order)"""
    nf = fine_prim.shape[1]
    nc = nf // r
    out = np.zeros((3, 16, nc**3))
    blk = fine_prim.reshape(NVAR, nc, r, nc, r, nc, r)  # var, kz, z, jy, y, ix, x
    for d in range(3):
        ax = {0: 6, 1: 4, 2: 2}[d]  # fine-offset axis of direction d
        other = [a for a in (2, 4, 6) if a != ax]
        red = tuple(o - (1 if o > ax else 0) for o in other)

        def layer(i):
            return np.take(blk, i, axis=ax).mean(axis=red)

        if r > 1:
            mf = 1.5 * layer(0) - 0.5 * layer(1)
            ml = 1.5 * layer(r - 1) - 0.5 * layer(r - 2)
        else:
            mf = ml = layer(0)
        out[d, :8] = _rotate_vars(mf, d).reshape(NVAR, -1)
        out[d, 8:] = _rotate_vars(ml, d).reshape(NVAR, -1)
    return out


def targets(coarse_prim, faces, d, gamma):
    """normalised correction targets [ncell, 16] of direction d"""
    vm, vp = plm_states(coarse_prim, d)
    sc = var_scale(_rotate_vars(coarse_prim, d), gamma).reshape(NVAR, -1)
    t = np.concatenate([(faces[d, :8] - vm) / sc, (faces[d, 8:] - vp) / sc], axis=0)
    return t.T


def downsample(fine_prim, fine_faces, r, gamma):
    """fine prim[8, nf, nf, nf] + faces [3][...] (left faces, compact periodic:
    faces[d] has the shape of the cells) -> coarse (prim[8, nc, nc, nc],
    faces[3, nc, nc, nc])"""
    g1 = gamma - 1.0
    rho = fine_prim[RHO]
    v = fine_prim[VX:VX + 3]
    B = fine_prim[BX:BX + 3]
    E = fine_prim[PRS] / g1 + 0.5 * rho * (v * v).sum(0) + 0.5 * (B * B).sum(0)
    nf = rho.shape[0]
    nc = nf // r

    def cavg(a):
        return a.reshape(nc, r, nc, r, nc, r).mean(axis=(1, 3, 5))

    U_rho = cavg(rho)
    U_m = np.stack([cavg(rho * v[k]) for k in range(3)])
    U_E = cavg(E)
    cf = np.zeros((3, nc, nc, nc))
    for d in range(3):
        f = fine_faces[d]
        # faces on coarse faces: fine index along d multiple of r
        sl = [slice(None)] * 3
        sl[2 - d] = slice(0, nf, r)
        sub = f[tuple(sl)]  # nc along d, nf along the others
        if d == 0:
            cf[0] = sub.reshape(nc, r, nc, r, nc).mean(axis=(1, 3))
        elif d == 1:
            cf[1] = sub.reshape(nc, r, nc, nc, r).mean(axis=(1, 4))
        else:
            cf[2] = sub.reshape(nc, nc, r, nc, r).mean(axis=(2, 4))
    Bc = np.stack([0.5 * (cf[d] + np.roll(cf[d], -1, axis=2 - d)) for d in range(3)])
    prim = np.zeros((NVAR, nc, nc, nc))
    prim[RHO] = U_rho
    prim[VX:VX + 3] = U_m / U_rho
    prim[BX:BX + 3] = Bc
    prim[PRS] = g1 * (U_E - 0.5 * U_rho * (prim[VX:VX + 3] ** 2).sum(0) - 0.5 * (Bc * Bc).sum(0))
    return prim, cf
