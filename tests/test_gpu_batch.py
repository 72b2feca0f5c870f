"""Batched boxes (mhd_batch_*): many independent cubes of uneven edge, each
with its own dt, stepped together: the classes of edge 32, 48, 64, 96 and 128
by work-list launches (one launch per operator over all of them), every other
class with one launch per size class per operator.

Each box of a batch must take exactly the steps a single-box context takes on
it: bit for bit against mhd_step for both arithmetic policies, and bit for bit
against the oracle (C/mhd.c:59-124 restated) for the EXACT kernels.
"""
import numpy as np
import pytest

from util import bitwise_equal

pytestmark = pytest.mark.gpu


def single(mhd, u0, b0, n, nsteps, exact):
    with mhd.Context(n, n, n, exact=exact) as ctx:
        ctx.set_state(u0, b0)
        ctx.step(nsteps, cfl=0.7)
        u, b = ctx.get_state()
        t, dt, _ = ctx.time()
    return u, b, t, dt


def make_batch(mhd, boxes, exact):
    bt = mhd.Batch([x["n"] for x in boxes], exact=exact)
    ics = []
    for i, box in enumerate(boxes):
        u0, b0 = mhd.init_batch_box(box)
        bt.set_box(i, u0, b0)
        ics.append((u0, b0))
    return bt, ics


@pytest.mark.parametrize("exact", [False, True])
def test_batch_equals_single_box_steps(exact, mhd, cuda):
    # uneven edges: TMA-aligned classes, a ragged one (17, 30) and repeats
    cfg = mhd.batch_config(9, seed=3, edges=(16, 17, 30, 32, 48))
    cfg[0]["n"], cfg[1]["n"] = 17, 30
    bt, ics = make_batch(mhd, cfg, exact)
    with bt:
        bt.step(4)
        bt.sync()
        for i, box in enumerate(cfg):
            u, b = bt.get_box(i)
            t, dt = bt.time(i)
            su, sb, st, sdt = single(mhd, *ics[i], box["n"], 4, exact)
            assert bitwise_equal(u, su) and bitwise_equal(b, sb), (i, box)
            assert t == st and dt == sdt, (i, t, st)


def test_batch_exact_bitwise_vs_oracle(mhd, cuda, oracle32):
    cfg = mhd.batch_config(40, seed=11)
    sample = [0, 1, 2, 3, 5, 8]
    boxes = [cfg[i] for i in sample]
    # one box of each edge in the sample at most 64^3 keeps the oracle within seconds
    for x, n in zip(boxes, (32, 48, 64, 32, 48, 32)):
        x["n"] = n
    bt, ics = make_batch(mhd, boxes, exact=True)
    with bt:
        bt.step(5)
        bt.sync()
        for i, box in enumerate(boxes):
            n = box["n"]
            u, b = bt.get_box(i)
            ou, ob, ot, _, _ = oracle32.strang(*ics[i], n, n, n, 5, 0.7)
            assert bitwise_equal(u, ou) and bitwise_equal(b, ob), (i, box)
            t, _ = bt.time(i)
            assert np.float32(t) == np.float32(ot)


def test_batch_boxes_keep_own_dt_and_graph_launches(mhd, cuda):
    cfg = mhd.batch_config(12, seed=5)
    bt, _ = make_batch(mhd, cfg, exact=False)
    with bt:
        ncls = bt.classes()
        assert ncls == len({x["n"] for x in cfg})
        bt.step(2)  # first step runs uncaptured (standalone calcfl), the second one is a graph
        c0 = bt.launch_count()
        bt.step(3)
        bt.sync()
        # 16 operators + the dt finalize: once for the work-list group, once per other class
        wl = bt.worklist_classes()
        assert wl == ncls  # the default edges all step in the work list
        assert bt.launch_count() - c0 == 3 * 17 * ((1 if wl else 0) + ncls - wl)
        dts = [bt.time(i)[1] for i in range(len(cfg))]
        assert all(np.isfinite(dts)) and min(dts) > 0
        assert len(set(dts)) > 1  # beta and Mach differ per box, so does dt


def test_batch_unloaded_box_is_refused(mhd, cuda):
    with mhd.Batch([32, 32]) as bt:
        u0, b0 = mhd.init_batch_box(dict(n=32, seed=1, beta=1.0, mach=0.5))
        bt.set_box(0, u0, b0)
        with pytest.raises(mhd.MhdError):
            bt.step(1)
        bt.set_box(1, u0, b0)
        bt.step(1)
        bt.sync()
        a, _ = bt.get_box(0)
        c, _ = bt.get_box(1)
        assert bitwise_equal(a, c)


def test_batch_device_buffers(mhd, cuda):
    torch = cuda
    box = dict(n=48, seed=2, beta=0.5, mach=0.8)
    u0, b0 = mhd.init_batch_box(box)
    du, db = torch.from_numpy(u0).cuda(), torch.from_numpy(b0).cuda()
    with mhd.Batch([48, 32]) as bt:
        bt.set_box(0, du, db)
        bt.set_box(1, *mhd.init_batch_box(dict(n=32, seed=3, beta=2.0, mach=0.3)))
        bt.step(2)
        bt.sync()
        ou, ob = torch.empty_like(du), torch.empty_like(db)
        bt.get_box_into(0, ou, ob)
        torch.cuda.synchronize()
        hu, hb = bt.get_box(0)
        assert bitwise_equal(ou.cpu().numpy(), hu) and bitwise_equal(ob.cpu().numpy(), hb)


def test_batch_x_walking_advect_exact_vs_oracle(mhd, cuda, oracle32):
    """Batched classes with the x-walking advectbyzx forced: several boxes of
    one class in one launch (the persistent CTAs of each box find it by
    blockIdx.z); EXACT bit for bit against the oracle."""
    from heterogeneous_mhd_gb300 import autotune
    cfg = mhd.batch_config(4, seed=13)
    for x, n in zip(cfg, (32, 64, 32, 64)):
        x["n"] = n
    try:
        autotune.apply({"advect.kernel": 4, "advect.xk": 4})
        bt, ics = make_batch(mhd, cfg, exact=True)
        with bt:
            bt.set_worklist(False)  # the global knobs shape the per-class launches only
            bt.step(3)
            bt.sync()
            for i, box in enumerate(cfg):
                n = box["n"]
                u, b = bt.get_box(i)
                ou, ob, _, _, _ = oracle32.strang(*ics[i], n, n, n, 3, 0.7)
                assert bitwise_equal(u, ou) and bitwise_equal(b, ob), (i, box)
    finally:
        autotune.apply({})


@pytest.mark.slow
def test_batch_large_classes_vs_oracle(mhd, cuda, oracle32):
    """The benched workload's two largest size classes (96^3 and 128^3 boxes,
    two of each with their own beta and Mach) inside a batch that also holds
    the smaller classes: sampled boxes bit for bit against the oracle with the
    EXACT kernels, and within the FAST one-step tolerance per field after one
    step with the production kernels."""
    from util import rel_l2_fields
    cfg = mhd.batch_config(10, seed=17)
    for x, n in zip(cfg, (96, 128, 96, 128, 32, 48, 64, 32, 48, 64)):
        x["n"] = n
    sample = [0, 1, 2, 3]
    for exact, nsteps in ((True, 2), (False, 1)):
        bt, ics = make_batch(mhd, cfg, exact=exact)
        with bt:
            bt.step(nsteps)
            bt.sync()
            for i in sample:
                n = cfg[i]["n"]
                u, b = bt.get_box(i)
                ou, ob, ot, _, _ = oracle32.strang(*ics[i], n, n, n, nsteps, 0.7)
                if exact:
                    assert bitwise_equal(u, ou) and bitwise_equal(b, ob), (i, cfg[i])
                    assert np.float32(bt.time(i)[0]) == np.float32(ot)
                else:
                    e = rel_l2_fields(u, b, ou, ob)
                    assert max(e.values()) <= 1e-5, (i, e)


def test_batch_per_edge_launch_shapes(mhd, cuda):
    """Launch-shape knobs set for one edge only (mhd_batch_tune_edge) change
    the kernels' shapes, not the results: the FAST boxes stay bit for bit
    those of the planner's shapes, and a knob for an edge the batch does not
    hold is refused."""
    cfg = mhd.batch_config(6, seed=5, edges=(32, 64))
    ref, ics = make_batch(mhd, cfg, exact=False)
    with ref:
        ref.step(3)
        ref.sync()
        want = [ref.get_box(i) for i in range(len(cfg))]
    bt, _ = make_batch(mhd, cfg, exact=False)
    with bt:
        edges = sorted({x["n"] for x in cfg})
        bt.tune_edge(edges[0], "advect.kernel", 3)
        bt.tune_edge(edges[0], "advect.K", 4)
        bt.tune_edge(edges[-1], "advect.J", 1)
        bt.tune_edge(edges[-1], "fluidx.threads", 128)
        with pytest.raises(mhd.MhdError):
            bt.tune_edge(40, "advect.K", 4)
        bt.step(3)
        bt.sync()
        for i in range(len(cfg)):
            u, b = bt.get_box(i)
            assert bitwise_equal(u, want[i][0]) and bitwise_equal(b, want[i][1]), i


@pytest.mark.parametrize("worklist", [False, True])
@pytest.mark.parametrize("exact", [False, True])
def test_batch_side_array_class_equals_single_box(exact, worklist, mhd, cuda):
    """Classes of 128^3 and 96^3 boxes run the plain step with the (rho, m_x)
    side array and the warp-per-pencil advectbyzx over all their boxes in one
    launch (128: one tensor map over the boxes' side arrays; 96: 3 cells per
    lane, bulk copies of the side-array pencils), per class or in the work
    list: each box bit for bit the single-box step, which uses the same
    kernels on one box."""
    cfg = mhd.batch_config(6, seed=21, edges=(128, 96, 64))
    for x, n in zip(cfg, (128, 128, 64, 128, 96, 96)):
        x["n"] = n
    bt, ics = make_batch(mhd, cfg, exact)
    with bt:
        bt.set_worklist(worklist)
        bt.step(2)
        bt.sync()
        for i, box in enumerate(cfg):
            u, b = bt.get_box(i)
            t, dt = bt.time(i)
            su, sb, st, sdt = single(mhd, *ics[i], box["n"], 2, exact)
            assert bitwise_equal(u, su) and bitwise_equal(b, sb), (i, box["n"])
            assert t == st and dt == sdt, (i, t, st)


@pytest.mark.parametrize("exact", [False, True])
def test_worklist_equals_per_class_launches(exact, mhd, cuda):
    """The work-list launches (one launch per operator over the classes of
    edge 32, 48, 64, 96 and 128; a class of edge 40 keeps its own launches)
    give every box the bits of one launch per class and operator, on the same
    initial states, after three steps; the whole work-list step is 17
    launches."""
    cfg = mhd.batch_config(9, seed=29)
    for x, n in zip(cfg, (128, 96, 64, 48, 32, 32, 48, 40, 64)):
        x["n"] = n
    ref, ics = make_batch(mhd, cfg, exact)
    with ref:
        ref.set_worklist(False)
        assert ref.worklist_classes() == 0
        ref.step(3)
        ref.sync()
        want = [ref.get_box(i) for i in range(len(cfg))]
        want_t = [ref.time(i) for i in range(len(cfg))]
    bt, _ = make_batch(mhd, cfg, exact)
    with bt:
        assert bt.worklist_classes() == 5 and bt.classes() == 6
        bt.step(2)
        c0 = bt.launch_count()
        bt.step(1)
        bt.sync()
        assert bt.launch_count() - c0 == 17 + 17  # the work list + the class of edge 40
        for i in range(len(cfg)):
            u, b = bt.get_box(i)
            assert bitwise_equal(u, want[i][0]) and bitwise_equal(b, want[i][1]), (i, cfg[i]["n"])
            assert bt.time(i) == want_t[i], i


def test_worklist_switch_and_own_shapes(mhd, cuda):
    """Switching the work list off and on between steps, and a class leaving it
    when given its own launch shapes, change only the launches: the FAST boxes
    stay bit for bit those of an uninterrupted work-list run."""
    cfg = mhd.batch_config(6, seed=31, edges=(32, 64, 96))
    ref, ics = make_batch(mhd, cfg, exact=False)
    with ref:
        ref.step(4)
        ref.sync()
        want = [ref.get_box(i) for i in range(len(cfg))]
    bt, _ = make_batch(mhd, cfg, exact=False)
    with bt:
        nw = bt.worklist_classes()
        bt.step(1)
        bt.set_worklist(False)
        bt.step(1)
        bt.set_worklist(True)
        edge = cfg[0]["n"]
        bt.tune_edge(edge, "advect.K", 4)
        assert bt.worklist_classes() == nw - 1
        bt.step(1)
        bt.tune_edge(edge, "advect.K", -1)
        assert bt.worklist_classes() == nw
        bt.step(1)
        bt.sync()
        for i in range(len(cfg)):
            u, b = bt.get_box(i)
            assert bitwise_equal(u, want[i][0]) and bitwise_equal(b, want[i][1]), i
