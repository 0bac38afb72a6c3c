"""Invariants of the reference algorithm, checked on the CPU oracle.

The reference's golden dumps are absent, so beside the pins to the
reference's own kernels (test_oracle_pin.py) the oracle is held to the
properties the exact scheme has:
* constrained transport keeps div B at round-off (checkDivB.hpp:14-68);
* a periodic box conserves mass, momentum and total energy to round-off
  (the flux-difference update, calcRightHandSide.hpp:333-550);
* the directional sweeps are interchangeable: a state with two axes swapped
  (vector components swapped with them) evolves into the swapped result;
* the Orszag-Tang problem (test/MHD/OrszagTang/setup.cpp:31-50) is symmetric
  under the point reflection (x, y) -> (1 - x, 1 - y) with vectors reversed,
  and stays so.
The last two hold to round-off only: mirrored states meet the Riemann solver
with left and right exchanged and the directional updates add in another
order."""
import numpy as np
import pytest

from idefix_gb300 import ic
from oracle.pyofx import Oracle

NG = 2


def _act(dims, n):
    """active cells of one variable's array ([1][nt1][nt0] in 2-D)"""
    return (Ellipsis,) + (slice(NG, NG + n),) * dims


def _ot(n=64):
    return ic.orszag_tang_2d(n, nghost=NG)


def _turb(n=16):
    return ic.turbulence_3d(n, seed=2, nghost=NG, kmax=4)


def _run(dims, n, state, cycles, cfl):
    o = Oracle(dims, (n,) * dims, cfl=cfl)
    o.set_prim(*state)
    assert o.run(max_cycles=cycles) == 0
    return o


@pytest.mark.parametrize("dims,cycles", [(2, 100), (3, 20)])
def test_div_b_stays_at_round_off(oracle_lib, dims, cycles):
    n = 64 if dims == 2 else 16
    state = _ot(n) if dims == 2 else _turb(n)
    o = _run(dims, n, state, cycles, 0.6 if dims == 2 else 0.4)
    assert o.check_divb() < 1e-12


@pytest.mark.parametrize("dims,cycles", [(2, 100), (3, 20)])
def test_periodic_box_conserves_mass_momentum_energy(oracle_lib, dims, cycles):
    n = 64 if dims == 2 else 16
    state = _ot(n) if dims == 2 else _turb(n)
    o = Oracle(dims, (n,) * dims, cfl=0.6 if dims == 2 else 0.4)
    o.set_prim(*state)
    o.lib.ofx_set_boundaries(o.h)
    o.lib.ofx_prim_to_cons(o.h)
    U0 = o.get_cons()
    assert o.run(max_cycles=cycles) == 0
    U1 = o.get_cons()
    act = _act(dims, n)
    assert U0[0][act].size == n**dims
    for q in range(dims + 2):  # RHO, MX1..MXd, ENG
        s0, s1 = np.sum(U0[q][act]), np.sum(U1[q][act])
        assert abs(s1 - s0) <= 1e-13 * np.sum(np.abs(U0[q][act])), (q, s0, s1)


def _swap(dims, Vc, Vs, a, b):
    """swap grid axes a and b (0 = x), with the vector components along them"""
    ax = {0: -1, 1: -2, 2: -3}
    V = Vc.swapaxes(ax[a], ax[b]).copy()
    V[[1 + a, 1 + b]] = V[[1 + b, 1 + a]]
    bx = dims + 2
    V[[bx + a, bx + b]] = V[[bx + b, bx + a]]
    S = Vs.swapaxes(ax[a], ax[b]).copy()
    S[[a, b]] = S[[b, a]]
    return V, S


@pytest.mark.parametrize("dims,a,b,cycles", [(2, 0, 1, 100), (3, 0, 1, 20), (3, 0, 2, 20)])
def test_swapped_axes_give_the_swapped_result(oracle_lib, dims, a, b, cycles):
    n = 64 if dims == 2 else 16
    state = _ot(n) if dims == 2 else _turb(n)
    cfl = 0.6 if dims == 2 else 0.4
    o1 = _run(dims, n, state, cycles, cfl)
    o2 = _run(dims, n, _swap(dims, *state, a, b), cycles, cfl)
    t1, t2 = o1.get_time(), o2.get_time()
    assert t1[2] == t2[2] and t1[0] == pytest.approx(t2[0], rel=1e-13)
    V1 = o1.get_prim()[0]
    V2 = _swap(dims, *o2.get_prim(), a, b)[0]
    act = _act(dims, n)
    for q in range(V1.shape[0]):
        scale = np.max(np.abs(V1[q][act]))
        assert np.max(np.abs(V1[q][act] - V2[q][act])) <= 1e-13 * scale, q


def test_orszag_tang_keeps_its_point_symmetry(oracle_lib):
    n = 64
    Vc, Vs = _ot(n)

    def reflect(V):  # cell-centred state under (x, y) -> (1 - x, 1 - y)
        R = V[..., ::-1, ::-1].copy()
        R[[1, 2, 4, 5]] *= -1.0
        return R

    act = _act(2, n)
    R0 = reflect(Vc)
    for q in range(6):
        assert np.max(np.abs(R0[q][act] - Vc[q][act])) < 1e-15
    V = _run(2, n, (Vc, Vs), 100, 0.6).get_prim()[0]
    R = reflect(V)
    for q in range(6):
        scale = np.max(np.abs(V[q][act]))
        assert np.max(np.abs(R[q][act] - V[q][act])) <= 1e-13 * scale, q


def test_orszag_tang_3d_keeps_div_b_and_conserves(oracle_lib):
    """the reference's 3-D benchmark problem (test/MHD/OrszagTang3D), its
    face field built from an edge potential: div B at round-off from the
    start, and after 10 cycles; mass, momentum and energy conserved"""
    n = (16, 32, 16)
    Vc, Vs = ic.orszag_tang_3d(*n)
    o = Oracle(3, n, cfl=0.9)
    o.set_prim(Vc, Vs)
    o.lib.ofx_set_boundaries(o.h)
    assert o.check_divb() < 1e-13
    o.lib.ofx_prim_to_cons(o.h)
    U0 = o.get_cons()
    assert o.run(max_cycles=10) == 0
    assert o.check_divb() < 1e-12
    U1 = o.get_cons()
    act = (Ellipsis, slice(NG, NG + n[2]), slice(NG, NG + n[1]), slice(NG, NG + n[0]))
    for q in range(5):
        s0, s1 = np.sum(U0[q][act]), np.sum(U1[q][act])
        assert abs(s1 - s0) <= 1e-13 * np.sum(np.abs(U0[q][act])), (q, s0, s1)
