"""The learned closure's kernels against the float64 oracle (oracle/closure_oracle.py).

BF16 operands with FP32 accumulation: each tolerance below is written next
to the comparison and is a few BF16 ulps (2^-8 relative) of the compared
quantity."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import closure_oracle as co  # noqa: E402

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def clos(mhd, cuda):
    from heterogeneous_mhd_gb300 import closure
    return closure


def to_bf16(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to("cuda").to(torch.bfloat16)


def to_f32(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to("cuda")


def bf_np(t):
    return t.float().cpu().numpy().astype(np.float64)


def features_input(rng, nb, n):
    x = np.zeros((nb, n, n, n, 16))
    x[..., :8] = rng.normal(size=(nb, n, n, n, 8))
    return x


def test_net_forward_loss_backward_vs_oracle(clos, cuda):
    torch = cuda
    rng = np.random.default_rng(0)
    nb, n = 2, 8
    params = clos.init_params(seed=3)
    params[-8:] = rng.normal(size=8) * 0.1  # non-zero head bias
    net = clos.ClosureNet(params)
    x = features_input(rng, nb, n)
    tgt = rng.normal(size=(nb, n, n, n, 8)) * 0.5
    xd, td = to_bf16(torch, x), to_bf16(torch, tgt)
    out = net.forward(xd, nb, n)
    net.loss(td, nb, n)
    net.backward(xd, nb, n)
    torch.cuda.synchronize()
    out = out.cpu().numpy().reshape(nb, n, n, n, 8)

    ps = clos.unflatten(params)
    ref, cache = co.net_forward(ps, co.bf16(x)[..., :8], round_bf16=True)
    tq = co.bf16(tgt)
    lref, dref = co.loss_and_grad(ref, tq[..., :5], tq[..., 5:])
    gref = co.net_backward([(co.bf16(w), b) for w, b in ps], cache, dref)

    assert rel(out, ref) < 2e-2                # BF16 activations through five layers
    assert abs(net.loss_value() - lref) < 2e-2 * lref
    dout = bf_np(net.dout).reshape(nb, n, n, n, 16)
    assert rel(dout[..., :8], dref) < 1e-2
    assert np.all(dout[..., 8:] == 0)
    g = clos.unflatten(net.grads_numpy())
    for li, ((gw, gb), (rw, rb)) in enumerate(zip(g, gref)):
        assert rel(gw, rw) < 5e-2, (li, rel(gw, rw))   # BF16 d z chain
        assert rel(gb, rb) < 5e-2, (li, rel(gb, rb))


def test_conv_kinds_vs_oracle(clos, cuda):
    """Each convolution kind alone: forward (GELU, head) and data gradient."""
    torch = cuda
    L = clos.cl()
    rng = np.random.default_rng(1)
    nb, n = 1, 16
    s = clos.stream_ptr()
    # hidden forward
    w = rng.normal(size=(32, 27, 32)) * 0.05
    b = rng.normal(size=32) * 0.1
    x = rng.normal(size=(nb, n, n, n, 32))
    wf = torch.empty(32 * 27 * 32, dtype=torch.bfloat16, device="cuda")
    wd = torch.empty_like(wf)
    wt = to_f32(torch, w)
    assert L.mhd_cl_pack(wt.data_ptr(), 32, 32, 27, 32, 32, wf.data_ptr(), wd.data_ptr(), s) == 0
    xd, bd = to_bf16(torch, x), to_f32(torch, b)
    a = torch.empty(nb * n ** 3 * 32, dtype=torch.bfloat16, device="cuda")
    z = torch.empty_like(a)
    assert L.mhd_cl_conv(clos.FWD_HID, xd.data_ptr(), wf.data_ptr(), bd.data_ptr(), a.data_ptr(), z.data_ptr(),
                         None, nb, n, s) == 0
    torch.cuda.synchronize()
    zr = co.conv3d(co.bf16(x), co.bf16(w).reshape(32, 3, 3, 3, 32), b)
    assert rel(bf_np(z).reshape(zr.shape), zr) < 8e-3        # one BF16 rounding of z
    assert rel(bf_np(a).reshape(zr.shape), co.gelu(co.bf16(zr))) < 1e-2
    # data gradient of the same layer: dx = conv^T(dz) * GELU'(zprev)
    dz = rng.normal(size=(nb, n, n, n, 32))
    zp = rng.normal(size=(nb, n, n, n, 32))
    dzd, zpd = to_bf16(torch, dz), to_bf16(torch, zp)
    dx = torch.empty_like(a)
    assert L.mhd_cl_conv(clos.DGRAD_HID, dzd.data_ptr(), wd.data_ptr(), None, dx.data_ptr(), None, zpd.data_ptr(),
                         nb, n, s) == 0
    torch.cuda.synchronize()
    dxr, _, _ = co.conv3d_backward(np.zeros_like(x), co.bf16(w).reshape(32, 3, 3, 3, 32), co.bf16(dz))
    dxr = dxr * co.gelu_grad(co.bf16(zp))
    assert rel(bf_np(dx).reshape(dxr.shape), dxr) < 1e-2


def test_wgrad_vs_oracle(clos, cuda):
    torch = cuda
    L = clos.cl()
    rng = np.random.default_rng(2)
    nb, n = 2, 8
    s = clos.stream_ptr()
    for kind, cin, cinr, coutp, coutr, ks in ((clos.WG_IN, 16, 8, 32, 32, 3), (clos.WG_HID, 32, 32, 32, 32, 3),
                                              (clos.WG_HEAD, 32, 32, 16, 8, 1)):
        a = rng.normal(size=(nb, n, n, n, cin))
        a[..., cinr:] = 0
        dz = rng.normal(size=(nb, n, n, n, coutp))
        dz[..., coutr:] = 0
        ad, dzd = to_bf16(torch, a), to_bf16(torch, dz)
        scr = torch.empty(int(L.mhd_cl_wgrad_scratch(kind, nb, n)) // 4 + 1, dtype=torch.float32, device="cuda")
        dw = torch.empty(coutr * ks ** 3 * cinr, dtype=torch.float32, device="cuda")
        assert L.mhd_cl_wgrad(kind, ad.data_ptr(), dzd.data_ptr(), scr.data_ptr(), dw.data_ptr(), nb, n, s) == 0
        torch.cuda.synchronize()
        w0 = np.zeros((coutr, ks, ks, ks, cinr))
        _, dwr, _ = co.conv3d_backward(co.bf16(a)[..., :cinr], w0, co.bf16(dz)[..., :coutr])
        assert rel(dw.cpu().numpy().reshape(dwr.shape), dwr) < 1e-4, kind  # FP32 sums of exact BF16 products


def test_filter_features_diff_vs_oracle(clos, mhd, cuda):
    torch = cuda
    L = clos.cl()
    s = clos.stream_ptr()
    u, b = mhd.init_turbulence(32, seed=4)
    ud, bd = to_f32(torch, u), to_f32(torch, b)
    uc = torch.empty(8 ** 3 * 5, dtype=torch.float32, device="cuda")
    bc = torch.empty(8 ** 3 * 3, dtype=torch.float32, device="cuda")
    assert L.mhd_cl_filter(ud.data_ptr(), bd.data_ptr(), 32, 4, uc.data_ptr(), bc.data_ptr(), s) == 0
    torch.cuda.synchronize()
    ur, br = co.box_filter(u, b, 32, 4)
    assert rel(uc.cpu().numpy(), ur) < 1e-6 and rel(bc.cpu().numpy(), br) < 1e-6
    assert mhd.host_divb_max(bc.cpu().numpy(), 8, 8, 8) < 1e-5
    mean = np.linspace(-0.1, 0.2, 8)
    inv = np.linspace(0.5, 2.0, 8)
    raw = torch.empty(8 ** 3 * 8, dtype=torch.float32, device="cuda")
    x = torch.empty(8 ** 3 * 16, dtype=torch.bfloat16, device="cuda")
    assert L.mhd_cl_features(uc.data_ptr(), bc.data_ptr(), 8, to_f32(torch, mean).data_ptr(),
                             to_f32(torch, inv).data_ptr(), raw.data_ptr(), x.data_ptr(), s) == 0
    torch.cuda.synchronize()
    xr = co.features(uc.cpu().numpy(), bc.cpu().numpy(), 8, mean, inv)
    assert rel(bf_np(x).reshape(xr.shape), xr) < 4e-3
    d = torch.empty(8 ** 3 * 8, dtype=torch.float32, device="cuda")
    assert L.mhd_cl_diff(uc.data_ptr(), bc.data_ptr(), uc.data_ptr(), bc.data_ptr(), 8, d.data_ptr(), s) == 0
    torch.cuda.synchronize()
    assert float(d.abs().max()) == 0.0


def test_correction_keeps_div_b_and_falls_back(clos, mhd, cuda):
    torch = cuda
    L = clos.cl()
    s = clos.stream_ptr()
    n = 16
    u, b = mhd.init_vortex(n, n, n, seed=5)
    rng = np.random.default_rng(5)
    out = rng.normal(size=(n, n, n, 8)) * 1e-3
    osc = np.array([1.0, 0.5, 0.5, 0.5, 2.0])
    bscale = 0.7
    ud, bd, od, sd = to_f32(torch, u), to_f32(torch, b), to_f32(torch, out), to_f32(torch, osc)
    ut = torch.empty_like(ud)
    bt = torch.empty_like(bd)
    flags = torch.zeros(4, dtype=torch.int32, device="cuda")
    esum = torch.zeros(8, dtype=torch.float64, device="cuda")
    fb = torch.zeros(1, dtype=torch.int64, device="cuda")
    args = (ut.data_ptr(), bt.data_ptr(), flags.data_ptr(), esum.data_ptr(), 1e-2, fb.data_ptr(), None, 0.0, s)
    assert L.mhd_cl_apply(ud.data_ptr(), bd.data_ptr(), od.data_ptr(), n, sd.data_ptr(), bscale, *args) == 0
    torch.cuda.synchronize()
    ur, br = co.apply_correction(u, b, out, n, osc, bscale)
    assert rel(ud.cpu().numpy(), ur) < 1e-6 and rel(bd.cpu().numpy(), br) < 1e-6
    assert int(fb.item()) == 0
    assert mhd.host_divb_max(bd.cpu().numpy(), n, n, n) < 1e-5  # CT update: div B at FP32 round-off
    # a correction whose full size breaks positivity is applied at the first of 1/2, 1/4 that keeps it
    part = out.copy()
    part[2, 2, 2, 0] = -1.2 / osc[0]  # rho ~ 1 - 1.2 < 0 at full size
    u_h, b_h = ud.cpu().numpy().copy(), bd.cpu().numpy().copy()
    expect = None
    for alpha in (1.0, 0.5, 0.25):
        uc, bc = co.apply_correction(u_h, b_h, part, n, osc, bscale, alpha=alpha)
        if uc.reshape(-1, 5)[:, 0].min() > 0 and co.pressure(uc, bc, n).min() > 0:
            expect = (alpha, uc, bc)
            break
    assert expect is not None and expect[0] < 1.0
    od_h = to_f32(torch, part)
    assert L.mhd_cl_apply(ud.data_ptr(), bd.data_ptr(), od_h.data_ptr(), n, sd.data_ptr(), bscale, *args) == 0
    torch.cuda.synchronize()
    assert rel(ud.cpu().numpy(), expect[1]) < 1e-6 and rel(bd.cpu().numpy(), expect[2]) < 1e-6
    assert int(fb.item()) == 0
    # a correction that makes rho negative even at a quarter of its size is refused
    bad = out.copy()
    bad[3, 4, 5, 0] = -10.0
    u1, b1 = ud.cpu().numpy().copy(), bd.cpu().numpy().copy()
    od2 = to_f32(torch, bad)
    assert L.mhd_cl_apply(ud.data_ptr(), bd.data_ptr(), od2.data_ptr(), n, sd.data_ptr(), bscale, *args) == 0
    torch.cuda.synchronize()
    assert int(fb.item()) == 1
    assert np.array_equal(ud.cpu().numpy(), u1) and np.array_equal(bd.cpu().numpy(), b1)


def test_adamw_vs_oracle(clos, cuda):
    torch = cuda
    rng = np.random.default_rng(6)
    p, g, m, v = (rng.normal(size=1000) for _ in range(4))
    v = np.abs(v)
    pd, gd, md, vd = (to_f32(torch, a) for a in (p, g, m, v))
    for step in (1, 7):
        assert clos.cl().mhd_cl_adamw(pd.data_ptr(), gd.data_ptr(), md.data_ptr(), vd.data_ptr(), 1000, step, 1e-3,
                                      0.9, 0.999, 1e-8, 1e-4, clos.stream_ptr()) == 0
        p, m, v = co.adamw(p, g, m, v, step, 1e-3)
    torch.cuda.synchronize()
    assert rel(pd.cpu().numpy(), p) < 1e-6 and rel(md.cpu().numpy(), m) < 1e-6 and rel(vd.cpu().numpy(), v) < 1e-6


def test_training_fits_a_teacher(clos, cuda):
    """AdamW on the kernels' gradients fits targets made by a random teacher net."""
    torch = cuda
    rng = np.random.default_rng(7)
    nb, n = 2, 16
    teacher = clos.ClosureNet(seed=11)
    student = clos.ClosureNet(seed=12)
    x = to_bf16(torch, features_input(rng, nb, n))
    out = teacher.forward(x, nb, n).cpu().numpy().reshape(nb, n, n, n, 8) * 10.0
    tgt = np.concatenate([out[..., :5], co.curl_faces(out[..., 5:])], axis=-1)
    td = to_bf16(torch, tgt)
    losses = []
    for it in range(300):
        student.forward(x, nb, n)
        student.loss(td, nb, n)
        student.backward(x, nb, n)
        student.adamw(lr=2e-3)
        if it % 50 == 0 or it == 299:
            losses.append(student.loss_value())
    assert losses[-1] < 0.1 * losses[0], losses


@pytest.mark.parametrize("kind", ["in", "hid", "dgrad"])
def test_tcgen05_conv_matches_mma_sync(kind, clos, cuda):
    """The tcgen05 kernel (n a multiple of 16) against the mma.sync kernel on the same operands."""
    torch = cuda
    L = clos.cl()
    rng = np.random.default_rng(8)
    nb, n = 2, 32
    cin = 16 if kind == "in" else 32
    s = clos.stream_ptr()
    w = rng.normal(size=(32, 27, 8 if kind == "in" else 32)) * 0.05
    wf = torch.empty(32 * 27 * cin, dtype=torch.bfloat16, device="cuda")
    wd = torch.empty(32 * 27 * cin, dtype=torch.bfloat16, device="cuda")
    assert L.mhd_cl_pack(to_f32(torch, w).data_ptr(), 32, w.shape[2], 27, 32, cin, wf.data_ptr(),
                         wd.data_ptr() if kind != "in" else None, s) == 0
    x = rng.normal(size=(nb, n, n, n, cin))
    if kind == "in":
        x[..., 8:] = 0
    xd = to_bf16(torch, x)
    bd = to_f32(torch, rng.normal(size=32) * 0.1)
    zp = to_bf16(torch, rng.normal(size=(nb, n, n, n, 32)))
    outs = []
    for tc in (1, 0, 2):  # warp-specialised tcgen05, mma.sync, two-buffer tcgen05
        L.mhd_cl_use_tcgen05(tc)
        y = torch.empty(nb * n ** 3 * 32, dtype=torch.bfloat16, device="cuda")
        z = torch.zeros_like(y)
        if kind == "dgrad":
            st = L.mhd_cl_conv(clos.DGRAD_HID, xd.data_ptr(), wd.data_ptr(), None, y.data_ptr(), None,
                               zp.data_ptr(), nb, n, s)
        else:
            st = L.mhd_cl_conv(clos.FWD_IN if kind == "in" else clos.FWD_HID, xd.data_ptr(), wf.data_ptr(),
                               bd.data_ptr(), y.data_ptr(), z.data_ptr(), None, nb, n, s)
        assert st == 0
        torch.cuda.synchronize()
        outs.append((bf_np(y), bf_np(z)))
    L.mhd_cl_use_tcgen05(1)
    assert L.mhd_cl_device_errors() == 0
    assert rel(outs[0][0], outs[1][0]) < 8e-3  # FP32 accumulation in two orders, one BF16 rounding
    if kind != "dgrad":
        assert rel(outs[0][1], outs[1][1]) < 8e-3
    # the two tcgen05 kernels issue the same MMAs in the same order: the same bits
    assert np.array_equal(outs[0][0], outs[2][0])
    if kind != "dgrad":
        assert np.array_equal(outs[0][1], outs[2][1])
