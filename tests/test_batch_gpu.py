"""Batched boxes through the C ABI (gch_batch_*).

FP32 batches without COOL_H, conduction, resistivity or passive scalars run
in grouped mode (table cooling and user spheres included): one launch per kernel of the step covers up to 64 boxes, the stage
kernels are persistent launches whose blocks pull (box, tile, z chunk) work
items from a device counter (or one block per item), and the z-march depth
and launch form come from the autotuner.  A box of a grouped batch must
compute what the same box computes alone (the grouped kernels run the
one-box kernel bodies), whatever depth the tuner picked and however the
boxes are chunked.  The FP32 units are compiled with multiply-add
contraction, and the compiler may contract a*b+c differently in the grouped
and the one-box instantiation of a body, so FP32 boxes are compared to the
single-domain run within a few FP32 roundings (`close`); an indexing or
chunking error shows up as an O(1) difference.  FP64 boxes (per-box mode,
no contraction) are compared bitwise."""
import dataclasses

import numpy as np
import pytest

from guacho_gb300 import params as P
from guacho_gb300 import problems

pytestmark = pytest.mark.gpu

# relative to the largest magnitude of each field; FP32 roundings after a
# few steps stay near 1e-7
RTOL = 1e-5


def close(a, ref, rtol=RTOL):
    """Per field: max |a - ref| <= rtol * max |ref|."""
    scale = np.maximum(np.abs(ref).reshape(-1, ref.shape[-1]).max(axis=0), 1e-30)
    err = np.abs(a - ref).reshape(-1, ref.shape[-1]).max(axis=0)
    return bool(np.all(err <= rtol * scale))


def _single(p, u, steps):
    from guacho_gb300.domain import Domain
    with Domain(p) as d:
        d.init(u)
        d.run(1e300, 1e300, max_steps=steps)
        return d.download(), d.time


@pytest.mark.parametrize("prec", [P.FP32_MIXED, P.FP32_KAHAN])
def test_grouped_batch_matches_single(gpu_lib, prec):
    from guacho_gb300.domain import Batch
    boxes = problems.batch_boxes(nbox=6, sizes=(16, 24, 32), precision=prec, seed=7)
    b = Batch([p for p, _ in boxes])
    for i, (_, u) in enumerate(boxes):
        b.upload(i, u)
    b.advance(3)
    b.advance(2)  # device-resident loop state carries over between calls
    tun = b.tuning()
    assert tun["grouped"] and tun["kz"] in tun["candidates"]
    # the autotuner searched depth x resident blocks per SM of the
    # persistent stage kernels and kept the fastest pair
    assert tun["blocks_per_sm"] in (0, 1, 2, 3)
    assert {b_ for _, b_ in tun["grid"]} == {0, 1, 2, 3}
    best = min(tun["grid"], key=tun["grid"].get)
    assert best == (tun["kz"], tun["blocks_per_sm"])
    times, iters = b.times()
    for i, (p, u) in enumerate(boxes):
        ref, t = _single(p, u, 5)
        assert iters[i] == 6 and times[i] == pytest.approx(t, rel=1e-6)
        assert close(b.download(i), ref), f"box {i}"
    b.close()


@pytest.mark.parametrize("prec", [P.FP32_MIXED, P.FP32_KAHAN])
def test_grouped_batch_ragged_boxes(gpu_lib, prec):
    """Boxes whose sides are not multiples of the 32 x 8 tile or of any
    z-march depth, grouped in one launch per kernel."""
    from guacho_gb300.domain import Batch
    dims = [(37, 19, 11), (13, 29, 7), (33, 9, 17), (5, 40, 3)]
    boxes = [problems.orszag_tang(*d, precision=prec) for d in dims]
    b = Batch([p for p, _ in boxes])
    for i, (_, u) in enumerate(boxes):
        b.upload(i, u)
    b.advance(4)
    assert b.tuning()["grouped"]
    for i, (p, u) in enumerate(boxes):
        ref, _ = _single(p, u, 4)
        assert close(b.download(i), ref), f"box {dims[i]}"
    b.close()


@pytest.mark.parametrize("prec", [P.FP32_MIXED, P.FP32_KAHAN])
def test_grouped_batch_wind_cooling(gpu_lib, prec):
    """Boxes of the hydro wind problem (HLLC, outflow, table cooling, two
    user spheres re-imposed at every boundary call) grouped: the stage-1
    fluxes and the CFL pass read the stored primitives, cooling and the
    ghost-shell primitives run after the stage-2 update, the spheres after
    every ghost fill -- each box as it runs alone.  The boxes differ in size,
    star density and wind speed."""
    from guacho_gb300.domain import Batch
    boxes = []
    for n, dens, vscale in ((16, 1.0, 1.0), (20, 2.0, 0.5), (24, 0.5, 1.5)):
        p, u = problems.wind_cooling(n, precision=prec)
        star = p.spheres[0]
        sph = [dataclasses.replace(star, dens=dens, vwind=star.vwind * vscale), p.spheres[1]]
        boxes.append((p.replace(spheres=sph), u))
    b = Batch([p for p, _ in boxes])
    for i, (_, u) in enumerate(boxes):
        b.upload(i, u)
    b.advance(3)
    b.advance(2)
    assert b.tuning()["grouped"]
    for i, (p, u) in enumerate(boxes):
        ref, _ = _single(p, u, 5)
        assert close(b.download(i), ref), f"box {i}"
    b.close()


def test_grouped_batch_more_boxes_than_one_launch(gpu_lib):
    """70 small boxes: two launches per kernel (64 + 6 boxes)."""
    from guacho_gb300.domain import Batch
    boxes = problems.batch_boxes(nbox=70, sizes=(8, 12), precision=P.FP32_KAHAN, seed=3)
    b = Batch([p for p, _ in boxes])
    for i, (_, u) in enumerate(boxes):
        b.upload(i, u)
    b.advance(4)
    for i in (0, 31, 63, 64, 69):
        p, u = boxes[i]
        ref, _ = _single(p, u, 4)
        assert close(b.download(i), ref), f"box {i}"
    b.close()


def test_grouped_batch_hydro_mixed_boundaries(gpu_lib):
    """Hydro HLLC (neq 5, the CFL reduction runs inside every step) with
    different boundary kinds and sizes per box."""
    from guacho_gb300.domain import Batch
    boxes = []
    for n, bc in ((12, P.BC_PERIODIC), (20, P.BC_OUTFLOW), (16, P.BC_CLOSED)):
        p, u = problems.orszag_tang(n, n, 8)
        p = p.replace(mhd=False, riemann_solver=P.SOLVER_HLLC, enable_flux_cd=False,
                      precision=P.FP32_MIXED, bc_left=bc, bc_right=bc, bc_bottom=bc,
                      bc_top=bc)
        boxes.append((p, np.ascontiguousarray(u[..., :5])))
    b = Batch([p for p, _ in boxes])
    for i, (_, u) in enumerate(boxes):
        b.upload(i, u)
    b.advance(4)
    assert b.tuning()["grouped"]
    for i, (p, u) in enumerate(boxes):
        ref, _ = _single(p, u, 4)
        assert close(b.download(i), ref), f"box {i}"
    b.close()


def test_fp64_batch_runs_per_box(gpu_lib):
    from guacho_gb300.domain import Batch
    boxes = problems.batch_boxes(nbox=2, sizes=(12,), precision=P.FP64, seed=5)
    b = Batch([p for p, _ in boxes])
    for i, (_, u) in enumerate(boxes):
        b.upload(i, u)
    b.advance(2)
    assert b.tuning() == {"grouped": False, "kz": -1, "blocks_per_sm": -1, "candidates": {},
                          "grid": {}}
    for i, (p, u) in enumerate(boxes):
        ref, _ = _single(p, u, 2)
        assert np.array_equal(b.download(i), ref)
    b.close()


@pytest.mark.parametrize("prec", [P.FP64, P.FP32_MIXED, P.FP32_KAHAN])
def test_z_march_depth_does_not_change_results(gpu_lib, prec):
    """Every plane is computed by the same code whatever the depth of the
    block's z march: 5 steps with kz = 1, 3 and 16 agree bitwise."""
    from guacho_gb300.domain import Domain
    p, u0 = problems.turbulence(20, seed=4)
    p = p.replace(precision=prec)
    outs = []
    for kz in (1, 3, 16):
        with Domain(p) as d:
            d.init(u0)
            d.kz = kz
            assert d.kz == kz
            d.run(1e300, 1e300, max_steps=5)
            outs.append(d.download())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


def test_autotune_keeps_state_and_picks_a_candidate(gpu_lib):
    from guacho_gb300.domain import Domain
    p, u0 = problems.turbulence(24, seed=9)
    p = p.replace(precision=P.FP32_KAHAN)
    with Domain(p) as d:
        d.init(u0)
        before = d.download()
        cand = d.autotune()
        assert d.kz in cand and all(ms > 0 for ms in cand.values())
        assert np.array_equal(d.download(), before)
        assert d.step_info() == (0, 0)
        d.run(1e300, 1e300, max_steps=3)
        tuned = d.download()
    with Domain(p) as d:
        d.init(u0)
        d.run(1e300, 1e300, max_steps=3)
        assert np.array_equal(d.download(), tuned)
