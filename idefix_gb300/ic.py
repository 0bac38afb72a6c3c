"""Initial conditions for the hot-path workloads, in the reference layout.

Every generator returns ``(Vc, Vs)`` as float64 numpy arrays laid out like
Idefix's ``Fluid::Vc`` / ``Fluid::Vs`` (LayoutRight, ghost zones included):

* ``Vc[nvar][nt2][nt1][nt0]`` with ``nt = n + 2*nghost`` (1 in unused dims)
* ``Vs[dims][nt2+ko][nt1+jo][nt0+io]`` (+1 in every active dimension)

Variable order follows src/idefix.hpp:74-108 (RHO, VX1..VXd, PRS, BX1..BXd).
Ghost cells are filled too; the first boundary pass of a cycle overwrites
them anyway, but the right-most face of each field component is an active
face and must hold a valid value.
"""
import math

import numpy as np


def grid_shapes(dims, n, nghost):
    n = list(n) + [1] * (3 - len(n))
    nt = [n[d] + 2 * nghost if d < dims else 1 for d in range(3)]
    ntv = [nt[d] + (1 if d < dims else 0) for d in range(3)]
    nvar = 2 * dims + 2
    return nvar, nt, ntv


def _coords(dims, n, nghost, xbeg, xend):
    """cell centres and left edges, as in gridHost.cpp:80-86"""
    xc, xl = [], []
    for d in range(3):
        if d < dims:
            dx = (xend[d] - xbeg[d]) / n[d]
            idx = np.arange(-nghost, n[d] + nghost, dtype=np.float64)
            xc.append(xbeg[d] + (idx + 0.5) * dx)
            xl.append(xbeg[d] + idx * dx)
        else:
            xc.append(np.zeros(1))
            xl.append(np.zeros(1))
    return xc, xl


def orszag_tang_2d(n=256, nghost=2, gamma=5.0 / 3.0):
    """2-D Orszag-Tang vortex on [0,1]^2 (test/MHD/OrszagTang/setup.cpp:25-62).

    Vs is set at every face index from the cell-centre coordinates of the
    same index, as the reference set-up does.
    """
    del gamma
    dims = 2
    nvar, nt, ntv = grid_shapes(dims, (n, n), nghost)
    xc, _ = _coords(dims, (n, n, 1), nghost, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    Vc = np.zeros((nvar, nt[2], nt[1], nt[0]))
    Vs = np.zeros((dims, ntv[2], ntv[1], ntv[0]))
    B0 = 1.0 / math.sqrt(4.0 * math.pi)
    x = xc[0][None, None, :]
    y = xc[1][None, :, None]
    Vc[0] = 25.0 / (36.0 * math.pi)
    Vc[3] = 5.0 / (12.0 * math.pi)
    Vc[1] = np.broadcast_to(-np.sin(2.0 * math.pi * y), Vc[1].shape)
    Vc[2] = np.broadcast_to(np.sin(2.0 * math.pi * x), Vc[2].shape)
    # faces: index (j,i) takes the centre coordinates x(i), y(j); the extra
    # face row/column beyond np_tot is a ghost face left at zero
    Vs[0, :, : nt[1], : nt[0]] = np.broadcast_to(-B0 * np.sin(2.0 * math.pi * y), (1, nt[1], nt[0]))
    Vs[1, :, : nt[1], : nt[0]] = np.broadcast_to(B0 * np.sin(4.0 * math.pi * x), (1, nt[1], nt[0]))
    return Vc, Vs


def rotor_2d(n=512, nghost=2):
    """MHD rotor on [-0.5,0.5]^2 (test/MHD/RotorCartesian/setup.cpp:17-60,
    idefix.ini: Roe, CFL 0.2, t_stop 0.15, outflow on all four sides): a
    dense disc (rho = 10, r < 0.1) spinning at omega = 20 with a linear taper
    to r = 0.115, in a uniform field B0 = 5 / sqrt(4 pi) along x, p = 1.

    Every cell and face index takes its cell-centre coordinates, as the
    reference set-up does; the extra face beyond np_tot stays zero (a ghost
    face, rebuilt by the boundary pass)."""
    dims = 2
    nvar, nt, ntv = grid_shapes(dims, (n, n), nghost)
    xc, _ = _coords(dims, (n, n, 1), nghost, (-0.5, -0.5, 0.0), (0.5, 0.5, 1.0))
    r0, r1, omega = 0.1, 0.115, 20.0
    B0 = 5.0 / math.sqrt(4.0 * math.pi)
    x = np.broadcast_to(xc[0][None, :], (nt[1], nt[0]))
    y = np.broadcast_to(xc[1][:, None], (nt[1], nt[0]))
    r = np.power(x * x + y * y, 0.5)
    f = (r1 - r) / (r1 - r0)
    inner, taper = r < r0, (r >= r0) & (r <= r1)
    rho = np.where(inner, 10.0, np.where(taper, 1.0 + 9.0 * f, 1.0))
    vphi = np.where(inner, omega * r, np.where(taper, f * omega * r0, 0.0))
    Vc = np.zeros((nvar, nt[2], nt[1], nt[0]))
    Vs = np.zeros((dims, ntv[2], ntv[1], ntv[0]))
    Vc[0, 0] = rho
    Vc[1, 0] = -y / r * vphi
    Vc[2, 0] = x / r * vphi
    Vc[3, 0] = 1.0
    Vs[0, :, : nt[1], : nt[0]] = B0
    return Vc, Vs


def shock_tube_2d(nx=800, ny=4, nghost=2):
    """MHD shock tube of test/MHD/sod (setup.cpp:30-55, idefix.ini: x in
    [0,100], Roe, gamma 1.66666666666667, CFL 0.8, t_stop 10, outflow in x):
    rho, p = 1, 1 for x < 50 and 0.125, 0.1 beyond, v = 0, Bx = 0.75,
    By = +1 / -1.  The reference runs it in 1-D with two components; here
    it is a 2-D block uniform in y (periodic, ny cells of the same width),
    so the y-derivatives vanish and By is a face field evolved by CT."""
    dims = 2
    dx = 100.0 / nx
    nvar, nt, ntv = grid_shapes(dims, (nx, ny), nghost)
    xc, xl = _coords(dims, (nx, ny, 1), nghost, (0.0, 0.0, 0.0), (100.0, ny * dx, 1.0))
    left = np.broadcast_to((xc[0] < 50.0)[None, :], (nt[1], nt[0]))
    Vc = np.zeros((nvar, nt[2], nt[1], nt[0]))
    Vs = np.zeros((dims, ntv[2], ntv[1], ntv[0]))
    Vc[0, 0] = np.where(left, 1.0, 0.125)
    Vc[3, 0] = np.where(left, 1.0, 0.1)
    Vs[0, :, : nt[1], : nt[0]] = 0.75
    Vs[1, :, : nt[1], : nt[0]] = np.where(left, 1.0, -1.0)
    return Vc, Vs


SHOCK_TUBE_GAMMA = 1.66666666666667  # test/MHD/sod/idefix.ini


def shock_tube_domain(nx=800, ny=4):
    """(xbeg, xend) of shock_tube_2d: [0,100] x [0, ny dx], square cells"""
    return (0.0, 0.0, 0.0), (100.0, ny * (100.0 / nx), 1.0)


ROTOR_DOMAIN = ((-0.5, -0.5, 0.0), (0.5, 0.5, 1.0))  # (xbeg, xend) of rotor_2d


FIELD_LOOP_DOMAIN = ((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0))  # (xbeg, xend) of field_loop_3d


def field_loop_3d(nx=128, ny=2, nz=128, nghost=2):
    """Advection of a weak field loop (test/MHD/FieldLoop/setup.cpp:17-56,
    idefix.ini: [-1,1]^3, HLLD, CFL 0.2, t_stop 2, periodic): rho = p = 1,
    v = (1, 0, 1), and the face field of the vector potential
    A_y = A0 (R0 - r) for r = sqrt(x^2 + z^2) <= R0 (A0 = 1e-3, R0 = 0.3),
    evaluated at the cell centres of every cell index, through
    DataBlockHost::MakeVsFromAmag's Cartesian differences
    (dataBlockHost.cpp: Bx = -(A_y(k+1) - A_y(k)) / dz, Bz = (A_y(i+1) -
    A_y(i)) / dx, By = 0), so the discrete div B vanishes.  The reference
    runs it with one cell in y; here the y extent holds ny cells of the same
    state (uniform in y)."""
    dims = 3
    n = (nx, ny, nz)
    nvar, nt, ntv = grid_shapes(dims, n, nghost)
    xb, xe = FIELD_LOOP_DOMAIN
    xc, _ = _coords(dims, n, nghost, xb, xe)
    dx = [(xe[d] - xb[d]) / n[d] for d in range(3)]
    A0, R0 = 1.0e-3, 0.3
    x = xc[0][None, :]
    z = xc[2][:, None]
    r = np.sqrt(x * x + z * z)
    Ay2 = A0 * (R0 - r) * (r <= R0)                     # [nt2][nt0], the same for every j
    Vc = np.zeros((nvar, nt[2], nt[1], nt[0]))
    Vs = np.zeros((dims, ntv[2], ntv[1], ntv[0]))
    Vc[0] = 1.0
    Vc[1] = 1.0
    Vc[3] = 1.0
    Vc[4] = 1.0
    g = nghost
    # active faces (and the extra right one in every direction), as the
    # reference's loop over [beg, end + 1)
    ks, js, is_ = slice(g, g + nz + 1), slice(g, g + ny + 1), slice(g, g + nx + 1)
    k = np.arange(g, g + nz + 1)
    i = np.arange(g, g + nx + 1)
    kk = np.minimum(k + 1, nt[2] - 1)
    ii = np.minimum(i + 1, nt[0] - 1)
    dAz = Ay2[kk][:, i] - Ay2[k][:, i]                  # A_y(k+1) - A_y(k)
    dAx = Ay2[k][:, ii] - Ay2[k][:, i]                  # A_y(i+1) - A_y(i)
    bx = (0.0 + 1.0 / dx[1] * 0.0) - 1.0 / dx[2] * dAz
    bz = 1.0 / dx[0] * dAx - 1.0 / dx[1] * 0.0
    Vs[0, ks, js, is_] = bx[:, None, :]
    Vs[2, ks, js, is_] = bz[:, None, :]
    return Vc, Vs


def orszag_tang_3d(nx=32, ny=64, nz=32, nghost=2):
    """3-D Orszag-Tang vortex on the periodic unit box (test/MHD/OrszagTang3D:
    setup.cpp:213-258, idefix.ini: 32 x 64 x 32, HLLD, CFL 0.9, t_stop 0.2;
    the reference's published GPU benchmark problem at 128^3, run without
    tracers): rho = 25/(36 pi), p = 5/(12 pi), v = (-sin 2pi y,
    sin 2pi x + cos 2pi z, cos 2pi x), and the face field of the edge
    potential A = B0/(2 pi) (cos 2pi y, sin 2pi x, cos 2pi y + cos(4pi x)/2)
    (B0 = 1/sqrt(4 pi); every component evaluated at the left-edge
    coordinates of its index) through DataBlockHost::MakeVsFromAmag's
    Cartesian differences (dataBlockHost.cpp:198-213), on the faces
    [beg, end + 1) of every direction."""
    dims = 3
    n = (nx, ny, nz)
    nvar, nt, ntv = grid_shapes(dims, n, nghost)
    xc, xl = _coords(dims, n, nghost, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    dx = [1.0 / n[d] for d in range(3)]
    B0 = 1.0 / math.sqrt(4.0 * math.pi)
    tp = 2.0 * math.pi
    X, Y, Z = (lambda a: a[None, None, :]), (lambda a: a[None, :, None]), (lambda a: a[:, None, None])
    shape = (nt[2], nt[1], nt[0])
    Vc = np.zeros((nvar, nt[2], nt[1], nt[0]))
    Vc[0] = 25.0 / (36.0 * math.pi)
    Vc[4] = 5.0 / (12.0 * math.pi)
    Vc[1] = np.broadcast_to(-np.sin(tp * Y(xc[1])), shape)
    Vc[2] = np.broadcast_to(np.sin(tp * X(xc[0])) + np.cos(tp * Z(xc[2])), shape)
    Vc[3] = np.broadcast_to(np.cos(tp * X(xc[0])), shape)
    # edge potential on the np_tot^3 indices (the reference's extra index
    # np_tot is never read by the differences below)
    Ax = np.broadcast_to(B0 / tp * np.cos(tp * Y(xl[1])), shape)
    Ay = np.broadcast_to(B0 / tp * np.sin(tp * X(xl[0])), shape)
    Az = np.broadcast_to(B0 / tp * (np.cos(tp * Y(xl[1])) + np.cos(2.0 * tp * X(xl[0])) / 2.0), shape)
    g = nghost
    s = np.s_[g:g + nz + 1, g:g + ny + 1, g:g + nx + 1]
    si = np.s_[g:g + nz + 1, g:g + ny + 1, g + 1:g + nx + 2]
    sj = np.s_[g:g + nz + 1, g + 1:g + ny + 2, g:g + nx + 1]
    sk = np.s_[g + 1:g + nz + 2, g:g + ny + 1, g:g + nx + 1]
    Vs = np.zeros((dims, ntv[2], ntv[1], ntv[0]))
    Vs[(0,) + s] = (0.0 + 1 / dx[1] * (Az[sj] - Az[s])) - 1 / dx[2] * (Ay[sk] - Ay[s])
    Vs[(1,) + s] = -1 / dx[0] * (Az[si] - Az[s]) + 1 / dx[2] * (Ax[sk] - Ax[s])
    Vs[(2,) + s] = 1 / dx[0] * (Ay[si] - Ay[s]) - 1 / dx[1] * (Ax[sj] - Ax[s])
    return Vc, Vs


def orszag_tang_like_2d(n, mach=1.0, beta=10.0 / 3.0, nghost=2, gamma=5.0 / 3.0):
    """Orszag-Tang vortex with a chosen sonic Mach number and plasma beta.

    rho and p are the vortex's (sound speed sqrt(gamma p / rho) = 1 at
    gamma = 5/3); the velocity amplitude is mach times the sound speed and
    the field amplitude B0 = sqrt(2 p / beta) (beta = p / (B0^2 / 2)).
    mach = 1, beta = 10/3 is the standard vortex.
    """
    Vc, Vs = orszag_tang_2d(n, nghost)
    p = 5.0 / (12.0 * math.pi)
    cs = math.sqrt(gamma * p / (25.0 / (36.0 * math.pi)))
    Vc[1:3] *= mach * cs
    b_scale = math.sqrt(2.0 * p / beta) * math.sqrt(4.0 * math.pi)
    Vs *= b_scale
    return Vc, Vs


ENSEMBLE_SIZES = (64, 96, 128, 192, 256, 384, 512)


def ensemble_boxes(nbox=512, seed=0, sizes=ENSEMBLE_SIZES):
    """Seeded ensemble of Orszag-Tang-like boxes: size uniform over `sizes`
    (square boxes), sonic Mach uniform in [0.5, 2], beta log-uniform in
    [0.1, 10].  Returns a list of (n, mach, beta)."""
    rng = np.random.default_rng(seed)
    n = rng.choice(np.asarray(sizes), size=nbox)
    mach = rng.uniform(0.5, 2.0, size=nbox)
    beta = 10.0 ** rng.uniform(-1.0, 1.0, size=nbox)
    return [(int(n[b]), float(mach[b]), float(beta[b])) for b in range(nbox)]


def _gaussian_field(rng, shape, kmin, kmax, slope=-2.0):
    """Real Gaussian random field with power ~ k^slope on kmin <= |k| <= kmax
    (integer wavenumbers of a periodic box), unit rms."""
    nz, ny, nx = shape
    kz = np.fft.fftfreq(nz) * nz
    ky = np.fft.fftfreq(ny) * ny
    kx = np.fft.rfftfreq(nx) * nx
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    k = np.sqrt(KX**2 + KY**2 + KZ**2)
    amp = np.zeros_like(k)
    m = (k >= kmin) & (k <= kmax)
    amp[m] = k[m] ** (slope / 2.0)
    ph = rng.standard_normal(k.shape) + 1j * rng.standard_normal(k.shape)
    f = np.fft.irfftn(amp * ph, s=shape, axes=(0, 1, 2))
    f /= np.sqrt(np.mean(f**2))
    return f


def _fill_periodic_cells(a, dims, nghost):
    """copy active cells into the ghost zones of a cell-centred array"""
    g = nghost
    for d in range(dims):
        ax = a.ndim - 1 - d
        n = a.shape[ax] - 2 * g
        idx = [(i - g) % n + g for i in range(a.shape[ax])]
        a[...] = np.take(a, idx, axis=ax)
    return a


def _curl_edges_to_faces(A, dx, dims):
    """Face-centred B = curl A from edge-centred A on a periodic grid, with
    the stencil of DataBlockHost::MakeVsFromAmag (dataBlockHost.cpp:198-213).
    A[c][k][j][i] are active-grid arrays; returns B[c][k][j][i] (active faces).
    """
    Ax, Ay, Az = A
    dx1, dx2, dx3 = dx
    roll = lambda a, ax: np.roll(a, -1, axis=ax)  # a(index+1)
    Bx = 1 / dx2 * (roll(Az, 1) - Az) - 1 / dx3 * (roll(Ay, 0) - Ay)
    By = -1 / dx1 * (roll(Az, 2) - Az) + 1 / dx3 * (roll(Ax, 0) - Ax)
    Bz = 1 / dx1 * (roll(Ay, 2) - Ay) - 1 / dx2 * (roll(Ax, 1) - Ax)
    return Bx, By, Bz


def _faces_to_Vs(B, nghost, ntv):
    """place periodic active-face arrays (k,j,i) into the ghosted Vs layout,
    including ghost faces and the extra right face of each component"""
    dims = 3
    g = nghost
    Vs = np.zeros((dims, ntv[2], ntv[1], ntv[0]))
    n = B[0].shape  # (nz, ny, nx)
    kk = (np.arange(ntv[2]) - g) % n[0]
    jj = (np.arange(ntv[1]) - g) % n[1]
    ii = (np.arange(ntv[0]) - g) % n[2]
    for c in range(3):
        Vs[c] = B[c][np.ix_(kk, jj, ii)]
    return Vs


def turbulence_3d(n=256, seed=1, nghost=2, gamma=5.0 / 3.0, mach=1.0, b0=0.1, beta=10.0,
                  kmin=1, kmax=8):
    """3-D decaying MHD turbulence in the periodic unit box.

    rho = 1, p = 1/gamma, velocity a seeded Gaussian field with power ~ k^-2 on
    integer 1 <= |k| <= kmax scaled to rms Mach ``mach``, B = (b0,0,0) + curl A
    with A a Gaussian field of the same spectrum, discretised on edges so that
    div B = 0 to round-off, scaled so that the mean plasma beta is ``beta``.
    """
    dims = 3
    nvar, nt, ntv = grid_shapes(dims, (n, n, n), nghost)
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    cs = math.sqrt(gamma * (1.0 / gamma) / 1.0)
    v = [_gaussian_field(rng, shape, kmin, kmax) for _ in range(3)]
    vrms = math.sqrt(sum(np.mean(c**2) for c in v))
    v = [c * (mach * cs / vrms) for c in v]
    A = [_gaussian_field(rng, shape, kmin, kmax) for _ in range(3)]
    dx = (1.0 / n, 1.0 / n, 1.0 / n)
    Bp = _curl_edges_to_faces(A, dx, dims)
    p0 = 1.0 / gamma
    # scale the fluctuation so that <p> / <B^2/2> = beta
    b2_target = 2.0 * p0 / beta
    bfl2 = sum(np.mean(c**2) for c in Bp)
    s = math.sqrt(max(b2_target - b0 * b0, 1e-30) / bfl2)
    B = [Bp[0] * s + b0, Bp[1] * s, Bp[2] * s]
    Vc = np.zeros((nvar, nt[2], nt[1], nt[0]))
    g = nghost
    act = (slice(g, g + n),) * 3
    Vc[0][act] = 1.0
    Vc[1][act], Vc[2][act], Vc[3][act] = v
    Vc[4][act] = p0
    for q in range(5):
        _fill_periodic_cells(Vc[q], dims, g)
    Vs = _faces_to_Vs(B, g, ntv)
    return Vc, Vs


def low_beta_3d(n=384, seed=1, nghost=2, gamma=5.0 / 3.0, beta=1e-3, mach=0.3, drho=0.1,
                kmin=1, kmax=4):
    """Low-beta precision workload: rho = 1 + drho G (G a seeded Gaussian
    field, k^-2 on kmin <= |k| <= kmax, unit rms), uniform Bz = 1, pressure
    from beta (p = beta B^2 / 2), velocity a Gaussian field of the same
    spectrum at rms Mach ``mach`` (sound speed of the mean state)."""
    dims = 3
    nvar, nt, ntv = grid_shapes(dims, (n, n, n), nghost)
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    G = _gaussian_field(rng, shape, kmin, kmax)
    rho = 1.0 + drho * G
    p0 = beta * 0.5
    cs = math.sqrt(gamma * p0 / 1.0)
    v = [_gaussian_field(rng, shape, kmin, kmax) for _ in range(3)]
    vrms = math.sqrt(sum(np.mean(c**2) for c in v))
    v = [c * (mach * cs / vrms) for c in v]
    Vc = np.zeros((nvar, nt[2], nt[1], nt[0]))
    g = nghost
    act = (slice(g, g + n),) * 3
    Vc[0][act] = rho
    Vc[1][act], Vc[2][act], Vc[3][act] = v
    Vc[4][act] = p0
    for q in range(5):
        _fill_periodic_cells(Vc[q], dims, g)
    zero = np.zeros(shape)
    Vs = _faces_to_Vs((zero, zero, zero + 1.0), g, ntv)
    return Vc, Vs


def uniform_random_3d(n=16, seed=0, nghost=2, gamma=5.0 / 3.0):
    """small seeded 3-D state for parity tests (turbulence spectrum, kmax=4)"""
    return turbulence_3d(n=n, seed=seed, nghost=nghost, gamma=gamma, kmax=min(4, n // 2))


def linear_wave_3d(mode=1, nx=64, ny=32, nz=32, nghost=2, gamma=5.0 / 3.0, epsilon=1.0e-6):
    """Oblique linear MHD wave of the reference's known-answer test
    (test/MHD/LinearWaveTest/setup.cpp; Gardiner & Stone 2008 eigenmodes) on
    [0,3]x[0,1.5]x[0,1.5].  mode: 1 fast, 2 Alfven, 3 slow, 4 entropy."""
    dims = 3
    n = (nx, ny, nz)
    nvar, nt, ntv = grid_shapes(dims, n, nghost)
    xbeg, xend = (0.0, 0.0, 0.0), (3.0, 1.5, 1.5)
    xc, xl = _coords(dims, n, nghost, xbeg, xend)
    RHO, VX1, VX2, VX3, PRS, BX1, BX2, BX3 = range(8)
    Bg = [0.0] * 8
    Bg[RHO], Bg[BX1], Bg[BX2], Bg[PRS] = 1.0, 1.0, 1.5, 1.0 / gamma
    R = [0.0] * 8
    absmode, sign = abs(mode), (1 if mode > 0 else -1)
    if absmode == 1:
        R0 = 1.0 / (2 * math.sqrt(5))
        R[RHO], R[VX1], R[VX2], R[BX2] = 2, sign * 4.0, -sign * 2.0, 4.0
        R[PRS] = (gamma - 1) * (9.0 - Bg[BX1] * R[BX1] - Bg[BX2] * R[BX2] - Bg[BX3] * R[BX3])
    elif absmode == 2:
        R0 = 1.0
        R[VX3], R[BX3] = -sign, 1.0
    elif absmode == 3:
        R0 = 1.0 / (2 * math.sqrt(5))
        R[RHO], R[VX1], R[VX2], R[BX2] = 4, 2 * sign, 4 * sign, -2.0
        R[PRS] = (gamma - 1) * (3.0 - Bg[BX1] * R[BX1] - Bg[BX2] * R[BX2] - Bg[BX3] * R[BX3])
    else:
        R0 = 0.5
        Bg[VX1] = 1
        R[RHO] = 2
        R[PRS] = (gamma - 1) * (1.0 - Bg[BX1] * R[BX1] - Bg[BX2] * R[BX2] - Bg[BX3] * R[BX3]
                                - Bg[VX1] * R[RHO] / 2.0)
    sinA, sinB = 2.0 / 3.0, 2.0 / math.sqrt(5.0)
    cosA, cosB = math.sqrt(1 - sinA * sinA), math.sqrt(1 - sinB * sinB)
    e1 = (cosA * cosB, cosA * sinB, sinA)
    e2 = (-sinB, cosB, 0.0)
    e3 = (-sinA * cosB, -sinA * sinB, cosA)
    X = xc[0][None, None, :]
    Y = xc[1][None, :, None]
    Z = xc[2][:, None, None]
    x1 = cosA * cosB * X + cosA * sinB * Y + sinA * Z
    phase = epsilon * np.cos(2.0 * math.pi * x1)
    Vc = np.zeros((nvar, nt[2], nt[1], nt[0]))
    Vc[RHO] = Bg[RHO] + R0 * R[RHO] * phase
    Vc[PRS] = Bg[PRS] + R0 * R[PRS] * phase
    for c, comp in ((VX1, 0), (VX2, 1), (VX3, 2)):
        Vc[c] = (Bg[VX1] * e1[comp] + Bg[VX2] * e2[comp] + Bg[VX3] * e3[comp]
                 + R0 * (R[VX1] * e1[comp] + R[VX2] * e2[comp] + R[VX3] * e3[comp]) * phase)

    def vecpot(xa, ya, za):
        x1 = cosA * cosB * xa + cosA * sinB * ya + sinA * za
        x2 = -sinB * xa + cosB * ya
        ph = epsilon * np.sin(2.0 * math.pi * x1) / (2.0 * math.pi)
        A1 = 0.0
        A2 = Bg[BX3] * x1 + R0 * R[BX3] * ph
        A3 = -(Bg[BX2] * x1 + R0 * R[BX2] * ph) + Bg[BX1] * x2
        return A1, A2, A3

    g = nghost
    dx = tuple((xend[d] - xbeg[d]) / n[d] for d in range(3))
    # the potential of the uniform field is not periodic (terms linear in
    # x1, x2), so the curl is taken on a grid extended by one cell
    B = _curl_nonperiodic(dx, xbeg, vecpot, e1, e2, e3, n)
    Vs = _faces_to_Vs(B, g, ntv)
    return Vc, Vs


def _curl_nonperiodic(dx, xbeg, vecpot, e1, e2, e3, n):
    """curl of the edge potential, evaluating A one cell beyond the domain
    directly rather than by wrap-around (the potential of a uniform field is
    not periodic, its curl is)."""
    nx, ny, nz = n
    def edge(comp, xs, ys, zs):
        A1, A2, A3 = vecpot(xs, ys, zs)
        e = (e1, e2, e3)
        return A1 * e[0][comp] + A2 * e[1][comp] + A3 * e[2][comp]

    dx1, dx2, dx3 = dx
    # coordinates extended by one cell on the right
    xcE = [xbeg[d] + (np.arange(n[d] + 1) + 0.5) * dx[d] for d in range(3)]
    xlE = [xbeg[d] + np.arange(n[d] + 1) * dx[d] for d in range(3)]
    X, Y, Z = (lambda a: a[None, None, :]), (lambda a: a[None, :, None]), (lambda a: a[:, None, None])
    AxE = edge(0, X(xcE[0]), Y(xlE[1]), Z(xlE[2]))  # (nz+1, ny+1, nx+1)
    AyE = edge(1, X(xlE[0]), Y(xcE[1]), Z(xlE[2]))
    AzE = edge(2, X(xlE[0]), Y(xlE[1]), Z(xcE[2]))
    shp = (nz + 1, ny + 1, nx + 1)
    AxE, AyE, AzE = (np.broadcast_to(a, shp) for a in (AxE, AyE, AzE))
    s = np.s_[:nz, :ny, :nx]
    sj = np.s_[:nz, 1:ny + 1, :nx]
    sk = np.s_[1:nz + 1, :ny, :nx]
    si = np.s_[:nz, :ny, 1:nx + 1]
    Bx = 1 / dx2 * (AzE[sj] - AzE[s]) - 1 / dx3 * (AyE[sk] - AyE[s])
    By = -1 / dx1 * (AzE[si] - AzE[s]) + 1 / dx3 * (AxE[sk] - AxE[s])
    Bz = 1 / dx1 * (AyE[si] - AyE[s]) - 1 / dx2 * (AxE[sj] - AxE[s])
    return Bx, By, Bz
