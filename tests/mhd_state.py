"""Helpers shared by the tests: move between the ghosted reference layout and
the active region (cells and the faces that the scheme evolves)."""
import numpy as np


def active_slices(dims, n, ng):
    n = list(n) + [1] * (3 - len(n))
    return [slice(ng, ng + n[d]) if d < dims else slice(0, 1) for d in range(3)]


def extract(dims, n, ng, Vc, Vs):
    """-> (Vc_active[nvar,nz,ny,nx], [Vs_c[nz(+1),ny(+1),nx(+1)] for c])"""
    sl = active_slices(dims, n, ng)
    vc = np.ascontiguousarray(Vc[:, sl[2], sl[1], sl[0]])
    vs = []
    for c in range(dims):
        s = list(sl)
        s[c] = slice(ng, ng + n[c] + 1)
        vs.append(np.ascontiguousarray(Vs[c, s[2], s[1], s[0]]))
    return vc, vs


def embed(dims, n, ng, vc, vs):
    """active arrays -> ghosted arrays (ghosts zero: the first boundary pass
    of a cycle overwrites every ghost value before it is read)"""
    n = list(n) + [1] * (3 - len(n))
    nvar = 2 * dims + 2
    nt = [n[d] + 2 * ng if d < dims else 1 for d in range(3)]
    ntv = [nt[d] + (1 if d < dims else 0) for d in range(3)]
    Vc = np.zeros((nvar, nt[2], nt[1], nt[0]))
    Vs = np.zeros((dims, ntv[2], ntv[1], ntv[0]))
    sl = active_slices(dims, n, ng)
    Vc[:, sl[2], sl[1], sl[0]] = vc
    for c in range(dims):
        s = list(sl)
        s[c] = slice(ng, ng + n[c] + 1)
        Vs[c, s[2], s[1], s[0]] = vs[c]
    return Vc, Vs


def l1_rel(a, b):
    """L1-relative difference sum|a-b| / sum|b| (per variable if 4-D)"""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.sum(np.abs(b))
    return float(np.sum(np.abs(a - b)) / den) if den > 0 else float(np.sum(np.abs(a - b)))
