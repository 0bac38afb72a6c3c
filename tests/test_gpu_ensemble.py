"""The batched ensemble (idfx_ens_*): independent periodic boxes of uneven
sizes advanced by shared launches, each with its own CFL time step.

Every box must evolve exactly as the same box run alone through the
single-block entry points (GpuBlock, itself bit-identical to the reference),
so every comparison here is exact equality of the state, the time, the time
step and the cycle count: with and without the CUDA graph, after the
autotuner, with the divB / NaN diagnostics on, with boxes that stop at
tstop after different numbers of cycles, and with a box that fails; and
in the persistent mode (every chunk of cycles one cooperative launch, its
phases separated by a bounded grid barrier).
"""
import numpy as np
import pytest

import idefix_gb300 as ig
from idefix_gb300 import ic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from idefix_gb300 import build

    build.build_library()
    ig.load_library()


def _box2d(n, mach, beta, **kw):
    Vc, Vs = ic.orszag_tang_like_2d(n, mach=mach, beta=beta)
    cfg = dict(dims=2, n=(n, n), **kw)
    return cfg, Vc, Vs


def _single(cfg, Vc, Vs, tstop=-1.0, cycles=-1):
    blk = ig.GpuBlock(**cfg)
    blk.upload(Vc, Vs)
    rc = None
    try:
        blk.run(tstop=tstop, max_cycles=cycles)
    except (ig.IdefixError, RuntimeError) as exc:
        rc = exc
    out = blk.download()
    t, dt, nc = blk.get_time()
    blk.close()
    return out, (t, dt, nc), rc


def _ensemble(boxes, tstop=-1.0, cycles=-1, graph=True, autotune=False, schedule=None, persistent=False):
    ens = ig.Ensemble([b[0] for b in boxes])
    for k, (_, Vc, Vs) in enumerate(boxes):
        ens.upload(k, Vc, Vs)
    if schedule:
        ens.set_schedule(schedule)
    if autotune:
        ens.autotune(reps=2)
    err = None
    try:
        ens.run(tstop=tstop, max_cycles=cycles, graph=graph, persistent=persistent)
    except (ig.IdefixError, RuntimeError) as exc:
        err = exc
    res = [(ens.download(k), ens.get_time(k)) for k in range(len(boxes))]
    segs = [ens.segments(k) for k in range(len(boxes))]
    ens.close()
    return res, err, segs


def _mixed_boxes(**kw):
    kw.setdefault("first_dt", 1e-4)
    spec = [(16, 0.5, 0.1, 0.6), (32, 2.0, 10.0, 0.8), (24, 1.0, 1.0, 0.5), (16, 1.7, 0.3, 0.9),
            (40, 0.8, 4.0, 0.7)]
    return [_box2d(n, m, b, cfl=c, **kw) for n, m, b, c in spec]


def _assert_same(res, boxes, tstop=-1.0, cycles=-1):
    for k, (cfg, Vc, Vs) in enumerate(boxes):
        (vc1, vs1), (t1, dt1, nc1), _ = _single(cfg, Vc, Vs, tstop=tstop, cycles=cycles)
        (vc2, vs2), (t2, dt2, nc2, st2) = res[k]
        assert st2 == 0, f"box {k} status {st2}"
        assert (t2, dt2, nc2) == (t1, dt1, nc1), f"box {k}"
        assert np.array_equal(vc1, vc2), f"box {k}: Vc differs"
        assert np.array_equal(vs1, vs2), f"box {k}: Vs differs"


@pytest.mark.parametrize("graph", [True, False])
def test_ensemble_matches_single_boxes(graph):
    boxes = _mixed_boxes()
    res, err, _ = _ensemble(boxes, cycles=10, graph=graph)
    assert err is None
    _assert_same(res, boxes, cycles=10)


def test_ensemble_with_diagnostics_and_rk3():
    boxes = _mixed_boxes(log_period=3, check_nan_period=2, nstages=3)
    res, err, _ = _ensemble(boxes, cycles=9)
    assert err is None
    _assert_same(res, boxes, cycles=9)


def test_ensemble_tstop_boxes_stop_independently():
    # per-box CFL dt: the boxes reach tstop after different cycle counts
    boxes = _mixed_boxes(log_period=4, check_nan_period=5)
    res, err, _ = _ensemble(boxes, tstop=0.1)
    assert err is None
    counts = {r[1][2] for r in res}
    assert len(counts) > 1
    _assert_same(res, boxes, tstop=0.1)


def test_ensemble_autotune_and_schedule_keep_results():
    boxes = _mixed_boxes()
    res, err, segs = _ensemble(boxes, cycles=6, autotune=True, schedule="box_order")
    assert err is None
    assert all(s[0] in (2, 4, 8, 16, 32, 64) and s[1] in (2, 4, 8, 16, 32, 64) for s in segs)
    _assert_same(res, boxes, cycles=6)


def test_ensemble_3d_and_mixed_precision():
    boxes = []
    for n, seed in ((40, 1), (12, 2), (8, 3)):
        Vc, Vs = ic.turbulence_3d(n, seed=seed, kmax=3)
        boxes.append((dict(dims=3, n=(n, n, n), cfl=0.6, precision="mixed"), Vc, Vs))
    res, err, _ = _ensemble(boxes, cycles=5)
    assert err is None
    _assert_same(res, boxes, cycles=5)


# The single mixed-precision block computes the corner EMFs and the face
# update in one fused pass over tiles of 32 x 8 edge columns marching
# segments of 32 layers (uct_contact, arithmetic and uct0; uct_hll and
# uct_hlld, whose corner EMFs read the face field, keep two passes); the
# ensemble keeps the two separate passes.  Equal bits check the single block
# against them, for every EMF average and for boxes whose edge counts end
# inside a tile and a segment (and reach a second segment).
@pytest.mark.parametrize("emf", ["uct_contact", "arithmetic", "uct0", "uct_hll", "uct_hlld"])
def test_fused_ct_pass_matches_separate_passes_3d(emf):
    boxes = []
    for n, seed in ((40, 4), (33, 5), (9, 6)):
        Vc, Vs = ic.turbulence_3d(n, seed=seed, kmax=3)
        boxes.append((dict(dims=3, n=(n, n, n), cfl=0.6, precision="mixed", emf=emf), Vc, Vs))
    res, err, _ = _ensemble(boxes, cycles=4)
    assert err is None
    _assert_same(res, boxes, cycles=4)


@pytest.mark.parametrize("emf,order", [("uct_contact", "limo3"), ("uct_hlld", "ppm"), ("uct0", "plm"),
                                       ("arithmetic", "plm")])
def test_fused_ct_pass_matches_separate_passes_2d(emf, order):
    ng = 3 if order == "ppm" else 2
    boxes = []
    for n, m, b, c in ((40, 1.2, 0.5, 0.6), (71, 0.7, 3.0, 0.8), (8, 1.0, 1.0, 0.5)):
        Vc, Vs = ic.orszag_tang_like_2d(n, mach=m, beta=b, nghost=ng)
        boxes.append((dict(dims=2, n=(n, n), cfl=c, precision="mixed", emf=emf, order=order, first_dt=1e-4),
                      Vc, Vs))
    res, err, _ = _ensemble(boxes, cycles=6)
    assert err is None
    _assert_same(res, boxes, cycles=6)


def test_ensemble_failed_box_leaves_the_others_running():
    boxes = _mixed_boxes()
    # a first_dt far above the CFL step fails at the end of the first cycle
    bad_cfg = dict(boxes[2][0], first_dt=1.0)
    boxes[2] = (bad_cfg, boxes[2][1], boxes[2][2])
    res, err, _ = _ensemble(boxes, cycles=7)
    assert isinstance(err, ig.IdefixError) and "box 2" in str(err)
    assert res[2][1][3] == ig.ERR_FIRST_DT
    good = [k for k in range(len(boxes)) if k != 2]
    _assert_same([res[k] for k in good], [boxes[k] for k in good], cycles=7)


def test_ensemble_rejects_mixed_schemes():
    cfg_a = dict(dims=2, n=(16, 16))
    cfg_b = dict(dims=2, n=(16, 16), solver="hll")
    with pytest.raises(ig.IdefixError):
        ig.Ensemble([cfg_a, cfg_b])


def test_ensemble_2d_mixed_precision():
    # the ensemble's FP32 x sweep is the per-thread march, the single block's
    # the warp-chunk sweep: equal bits check one against the other
    boxes = _mixed_boxes(precision="mixed")
    res, err, _ = _ensemble(boxes, cycles=6)
    assert err is None
    _assert_same(res, boxes, cycles=6)


# The single mixed block carries its state from stage to stage differently
# from the ensemble: its stage ends write the next stage's inputs (and leave
# the field part of Uc unstored), its last face update of a cycle writes the
# faces' Runge-Kutta begin copy, and its later stage begins and face fills
# pass over the ghosts alone.  Equal bits check those paths with the
# diagnostics on (the NaN check reads the primitives), RK3 (other stage
# weights) and boxes that stop at tstop after different cycle counts.
@pytest.mark.parametrize("kw,stop", [(dict(log_period=3, check_nan_period=2, nstages=3), dict(cycles=7)),
                                     (dict(log_period=4, check_nan_period=3), dict(tstop=0.05))])
def test_ensemble_mixed_precision_with_diagnostics_and_tstop(kw, stop):
    boxes = _mixed_boxes(precision="mixed", **kw)
    res, err, _ = _ensemble(boxes, **stop)
    assert err is None
    _assert_same(res, boxes, **stop)


def test_ensemble_with_shock_flattening():
    boxes = _mixed_boxes(shock_flattening=0.0)
    res, err, _ = _ensemble(boxes, cycles=8)
    assert err is None
    _assert_same(res, boxes, cycles=8)


def _persistent_cases():
    return {
        "plain": (_mixed_boxes(), dict(cycles=10)),
        "diagnostics_rk3": (_mixed_boxes(log_period=3, check_nan_period=2, nstages=3), dict(cycles=9)),
        "tstop": (_mixed_boxes(log_period=4, check_nan_period=5), dict(tstop=0.1)),
        "chunks": (_mixed_boxes(log_period=7, check_nan_period=11), dict(cycles=150)),
        "mixed_precision": (_mixed_boxes(precision="mixed"), dict(cycles=6)),
        "shock": (_mixed_boxes(shock_flattening=0.0), dict(cycles=8)),
    }


@pytest.mark.parametrize("case", ["plain", "diagnostics_rk3", "tstop", "chunks", "mixed_precision", "shock"])
def test_persistent_launch_matches_single_boxes(case):
    boxes, kw = _persistent_cases()[case]
    res, err, _ = _ensemble(boxes, persistent=True, **kw)
    assert err is None
    _assert_same(res, boxes, **kw)


def test_persistent_launch_3d_and_failed_box():
    boxes = []
    for n, seed in ((24, 1), (12, 2), (8, 3)):
        Vc, Vs = ic.turbulence_3d(n, seed=seed, kmax=3)
        boxes.append((dict(dims=3, n=(n, n, n), cfl=0.6), Vc, Vs))
    res, err, _ = _ensemble(boxes, cycles=5, persistent=True)
    assert err is None
    _assert_same(res, boxes, cycles=5)
    boxes = _mixed_boxes()
    boxes[2] = (dict(boxes[2][0], first_dt=1.0), boxes[2][1], boxes[2][2])
    res, err, _ = _ensemble(boxes, cycles=7, persistent=True)
    assert isinstance(err, ig.IdefixError) and "box 2" in str(err)
    assert res[2][1][3] == ig.ERR_FIRST_DT
    good = [k for k in range(len(boxes)) if k != 2]
    _assert_same([res[k] for k in good], [boxes[k] for k in good], cycles=7)


def test_persistent_launch_is_one_cooperative_launch():
    """the persistent mode's chunk is a single cooperative launch of all
    co-resident blocks (replayed from a CUDA graph where the capture of a
    cooperative launch is available; either way the results are equal)"""
    boxes = _mixed_boxes()
    ens = ig.Ensemble([b[0] for b in boxes])
    for k, (_, Vc, Vs) in enumerate(boxes):
        ens.upload(k, Vc, Vs)
    ens.run(max_cycles=3, persistent=True)
    blocks, graph = ens.persistent_info()
    ens.close()
    assert blocks >= 148
    assert graph in (True, False)
