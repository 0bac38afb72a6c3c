"""Learned interface-state correction: trainer and data preparation.

The network and its kernels live in csrc/learned.cu (C ABI idfx_mlp_*,
idfx_gpu_set_learned, idfx_learn_coarsen_device); this module drives them.
Device buffers are torch tensors (plumbing only: every computation on them
is one of the library's kernels, apart from dtype conversions and copies).
"""
import ctypes

import numpy as np

import idefix_gb300 as ig

NPARAM = 46352
NIN = 216
K1 = 224
NOUT = 16


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def init_params(seed=0, out_scale=0.0):
    """He-style initial parameters; the output layer starts at out_scale x
    (zero by default, so an untrained network makes no correction)."""
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((NIN, 128)) * np.sqrt(2.0 / NIN)
    W2 = rng.standard_normal((128, 128)) * np.sqrt(2.0 / 128)
    W3 = rng.standard_normal((128, NOUT)) * np.sqrt(2.0 / 128) * out_scale
    return np.concatenate([W1.ravel(), np.zeros(128), W2.ravel(), np.zeros(128), W3.ravel(),
                           np.zeros(NOUT)]).astype(np.float32)


def coarsen(Vc, Vs, nf, nghost, r, gamma=5.0 / 3.0):
    """Coarsen a 3-D periodic fine snapshot held in device tensors (reference
    layout, float64) by r: -> (prim [8,nc,nc,nc], faces [3,nc,nc,nc],
    targets [3,16,nc^3]) float64 device tensors."""
    import torch

    lib = ig.load_library()
    nc = nf // r
    prim = torch.empty((8, nc, nc, nc), dtype=torch.float64, device=Vc.device)
    faces = torch.empty((3, nc, nc, nc), dtype=torch.float64, device=Vc.device)
    tg = torch.empty((3, 16, nc * nc * nc), dtype=torch.float64, device=Vc.device)
    stream = torch.cuda.current_stream(Vc.device).cuda_stream
    rc = lib.idfx_learn_coarsen_device(_ptr(Vc), _ptr(Vs), nf, nghost, r, gamma, _ptr(prim), _ptr(faces),
                                       _ptr(tg), ctypes.c_void_p(stream))
    if rc != ig.OK:
        raise ig.IdefixError(f"idfx_learn_coarsen_device failed with status {rc}")
    return prim, faces, tg


def coarse_state(prim, faces, nghost=2):
    """compact coarse (prim, faces) -> ghosted host (Vc, Vs) for GpuBlock"""
    prim = prim.cpu().numpy() if hasattr(prim, "cpu") else np.asarray(prim)
    faces = faces.cpu().numpy() if hasattr(faces, "cpu") else np.asarray(faces)
    nc = prim.shape[1]
    g = nghost
    nt = nc + 2 * g
    Vc = np.zeros((8, nt, nt, nt))
    Vs = np.zeros((3, nt + 1, nt + 1, nt + 1))
    a = slice(g, g + nc)
    Vc[:, a, a, a] = prim
    for d in range(3):
        f = faces[d]
        # left faces of the active cells and the periodic last face
        ext = np.concatenate([f, np.take(f, [0], axis=2 - d)], axis=2 - d)
        sl = [a, a, a]
        sl[2 - d] = slice(g, g + nc + 1)
        Vs[d][tuple(sl)] = ext
    return Vc, Vs


class Trainer:
    """BF16 tensor-core trainer of the correction network (idfx_mlp_*)."""

    def __init__(self, max_batch=8192, params=None):
        self.lib = ig.load_library()
        h = ctypes.c_void_p()
        rc = self.lib.idfx_mlp_create(int(max_batch), None, ctypes.byref(h))
        if rc != ig.OK:
            raise ig.IdefixError(f"idfx_mlp_create failed with status {rc}")
        self.h = h
        self.max_batch = max_batch
        self._data = None
        self.set_params(init_params() if params is None else params)

    def close(self):
        if getattr(self, "h", None):
            self.lib.idfx_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc, what):
        if rc != ig.OK:
            raise ig.IdefixError(f"{what} failed with status {rc}")

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self.lib.idfx_mlp_set_params(self.h, _fp(p)), "idfx_mlp_set_params")

    def get_params(self):
        p = np.empty(NPARAM, dtype=np.float32)
        self._check(self.lib.idfx_mlp_get_params(self.h, _fp(p)), "idfx_mlp_get_params")
        return p

    def set_dataset(self, prims, targets, gamma=5.0 / 3.0):
        """prims float32 [S,8,nc,nc,nc], targets float32 [S,3,16,nc^3] (device)"""
        S, nc = prims.shape[0], prims.shape[2]
        self._data = (prims, targets)
        self._check(self.lib.idfx_mlp_set_dataset_device(self.h, _ptr(prims), _ptr(targets), S, nc, gamma),
                    "idfx_mlp_set_dataset_device")

    def train(self, steps, batch, lr=1e-3, lr_end=1e-5, seed=0):
        losses = np.zeros(max(steps, 1), dtype=np.float32)
        self._check(self.lib.idfx_mlp_train(self.h, steps, batch, lr, lr_end, seed, _fp(losses)), "idfx_mlp_train")
        return losses[:steps]

    def eval(self, batch, seed=12345):
        """(loss with the network, loss with no correction) on a random batch"""
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.idfx_mlp_eval(self.h, batch, seed, ctypes.byref(a), ctypes.byref(b)), "idfx_mlp_eval")
        return a.value, b.value

    def feature_range(self):
        lo = np.empty(NIN, dtype=np.float32)
        hi = np.empty(NIN, dtype=np.float32)
        self._check(self.lib.idfx_mlp_feature_range(self.h, _fp(lo), _fp(hi)), "idfx_mlp_feature_range")
        return lo, hi

    def batch(self, batch, seed=0, base=0):
        """one batch (X bfloat16 [batch, 224], T float32 [batch, 16]) on the device"""
        import torch

        X = torch.empty((batch, K1), dtype=torch.bfloat16, device="cuda")
        T = torch.empty((batch, NOUT), dtype=torch.float32, device="cuda")
        self._check(self.lib.idfx_mlp_batch_device(self.h, batch, seed, base, _ptr(X), _ptr(T)),
                    "idfx_mlp_batch_device")
        return X, T

    def grad(self, X, T):
        g = np.empty(NPARAM, dtype=np.float32)
        loss = ctypes.c_double()
        self._check(self.lib.idfx_mlp_grad_device(self.h, _ptr(X), _ptr(T), X.shape[0], _fp(g), ctypes.byref(loss)),
                    "idfx_mlp_grad_device")
        return g, loss.value

    def forward(self, X):
        import torch

        Y = torch.empty((X.shape[0], NOUT), dtype=torch.float32, device=X.device)
        self._check(self.lib.idfx_mlp_forward_device(self.h, _ptr(X), X.shape[0], _ptr(Y)),
                    "idfx_mlp_forward_device")
        return Y
