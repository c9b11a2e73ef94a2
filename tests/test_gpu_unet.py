"""U-Net kernels on the GPU against a plain PyTorch fp32 reference of the same
operation (bf16 inputs, fp32 accumulation; outputs compared after the kernel's
bf16 rounding)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BF16_TOL = 1e-2  # relative L2: bf16 output rounding is 2^-8 ~ 4e-3 per element


def conv_ref(x, w, b, relu):
    import torch

    # x: [N,H,W,Cin] bf16, w: [Cout,9,Cin] bf16 -> fp32 reference in NCHW
    xf = x.float().permute(0, 3, 1, 2)
    cout, _, cin = w.shape
    wf = w.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    y = torch.nn.functional.conv2d(xf, wf, b, padding=1)
    if relu:
        y = torch.relu(y)
    return y.permute(0, 2, 3, 1)


def run_conv(gb, x, w, b, relu, layout=0):
    import torch

    n, h, wd, cin = x.shape
    cout = w.shape[0]
    y = torch.zeros(n, h, wd, cout, dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    L = gb.lib()
    L.arecgb_conv3x3_bf16.argtypes = [C.c_void_p] * 4 + [C.c_int] * 7 + [C.c_void_p, C.c_void_p]
    rc = L.arecgb_conv3x3_bf16(x.data_ptr(), w.data_ptr(), b.data_ptr() if b is not None else None,
                               y.data_ptr(), n, h, wd, cin, cout, int(relu), layout,
                               err.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0, gb.last_error()
    assert int(err.item()) == 0
    return y


@pytest.mark.parametrize("cin,cout,shape", [(32, 32, (1, 16, 16)), (32, 64, (2, 8, 24)),
                                            (64, 128, (1, 32, 32)), (128, 256, (1, 12, 20)),
                                            (256, 32, (3, 9, 7))])
def test_conv3x3_matches_torch(gb, cin, cout, shape):
    import torch

    torch.manual_seed(cin + cout)
    n, h, wd = shape
    x = torch.randn(n, h, wd, cin, device="cuda").bfloat16()
    w = (torch.randn(cout, 9, cin, device="cuda") / (3 * cin ** 0.5)).bfloat16()
    b = torch.randn(cout, device="cuda") * 0.1
    ref = conv_ref(x, w, b, relu=True)
    errs = {}
    for layout in (0, 1):
        y = run_conv(gb, x, w, b, True, layout)
        errs[layout] = float((y.float() - ref).norm() / ref.norm())
    print("conv %d->%d %s: rel err layout0 %.2e layout1 %.2e" % (cin, cout, shape, errs[0], errs[1]))
    assert errs[0] < BF16_TOL


# Whole-network forward and gradients against the CPU oracle (oracle/unet_ref.py,
# FP64 autograd rounding activations and tensor-core weights to bf16 where the
# GPU stores bf16).
#
# Exact case: sparse weights (one +-1 or +-1/2 per output channel), zero
# biases, small-integer inputs and output gradients keep every activation and
# gradient exactly representable in bf16 and every sum exact in FP32, so the
# GPU must match the oracle to EXACT_TOL whatever the summation order: this
# pins indexing, concatenation, pooling, upsampling and the flipped weights.
#
# Random case: He-initialised weights.  Then rounding-boundary flips (FP32 on
# the GPU vs FP64 in the oracle) propagate through the network: the oracle
# itself moves by 0.3-0.5% between FP32 and FP64 accumulation.
# RAND_FWD_TOL / RAND_GRAD_TOL bound that statistical drift.
EXACT_TOL = 1e-6   # forward: the same bf16 values
EXACT_GRAD_TOL = 1e-5  # weight gradients: FP32 sums over all pixels, order differs
RAND_FWD_TOL = 3e-2
RAND_GRAD_TOL = 0.25


def _sparse_params(layers, nparams, rng):
    """Three nonzero weights per output channel, +-1/2 or +-1/4 (80% positive
    so activations survive the ReLUs), zero biases, output weights +-1.  The
    oracle gives identical results in FP32 and FP64 for these (every sum that
    is rounded to bf16 is exact), yet every layer gets nonzero gradients."""
    p = np.zeros(nparams)
    for l in layers:
        ci, co = l["cin"], l["cout"]
        if l["name"] == "out":
            p[l["w_off"]:l["w_off"] + ci] = rng.choice([-1.0, 1.0], size=ci)
            continue
        w = np.zeros((co, 9, ci))
        for _ in range(3):
            sign = np.where(rng.random(co) < 0.8, 1.0, -1.0)
            w[np.arange(co), rng.integers(0, 9, co), rng.integers(0, ci, co)] += (
                sign * rng.choice([0.5, 0.25], size=co))
        p[l["w_off"]:l["w_off"] + co * 9 * ci] = w.reshape(-1)
    return p


def _random_params(layers, nparams, rng):
    p = np.zeros(nparams)
    for l in layers:
        ci, co = l["cin"], l["cout"]
        if l["name"] == "out":
            p[l["w_off"]:l["w_off"] + ci] = 0.3 * rng.standard_normal(ci)
        else:
            n = co * 9 * ci
            p[l["w_off"]:l["w_off"] + n] = rng.standard_normal(n) * np.sqrt(2.0 / (9 * ci))
        p[l["b_off"]:l["b_off"] + co] = 0.05 * rng.standard_normal(co)
    return p.astype(np.float32).astype(np.float64)


def _compare(gb, size, batch, params, x, dout):
    import torch

    from oracle import unet_ref

    net = gb.UNet(size, batch, train=True, seed=1)
    assert (net.layers, net.nparams) == unet_ref.layer_table()
    net.set_params(torch.from_numpy(params.astype(np.float32)).cuda())
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    yd = torch.zeros_like(xd)
    net.forward(xd, yd)
    grads = torch.zeros(net.nparams, device="cuda")
    net.backward(torch.from_numpy(dout.astype(np.float32)).cuda(), grads)
    y_ref, g_ref = unet_ref.forward_and_grads(params, net.layers, net.nparams, x, dout)
    y, g = yd.cpu().numpy(), grads.cpu().numpy()
    e_fwd = np.linalg.norm(y - y_ref) / max(np.linalg.norm(y_ref - x), 1e-30)
    errs = {}
    for l in net.layers:
        n_w = l["cin"] if l["name"] == "out" else l["cout"] * 9 * l["cin"]
        for what, off, cnt in (("W", l["w_off"], n_w), ("b", l["b_off"], l["cout"])):
            a, b = g[off:off + cnt], g_ref[off:off + cnt]
            nb = np.linalg.norm(b)
            errs[l["name"] + "." + what] = (np.linalg.norm(a - b) / nb if nb > 0
                                            else float(np.linalg.norm(a)))
    return e_fwd, errs


@pytest.mark.parametrize("cin,cout,shape", [(32, 32, (1, 3, 128)), (64, 128, (2, 2, 256)),
                                            (256, 32, (1, 4, 128)), (128, 256, (1, 2, 128)),
                                            (32, 32, (2, 8, 256)), (64, 32, (1, 12, 128)),
                                            (32, 64, (2, 6, 128)), (128, 64, (1, 4, 256))])
def test_conv3x3_tma_path(gb, cin, cout, shape):
    """Widths that are multiples of 128 take the TMA path (layout 0): 32 output
    channels and heights divisible by 4, or 64 output channels and even heights,
    take the kernel that computes several rows per block (the image's first and
    last rows read zeros from outside it); the rest the one-row kernel.  Layout 2
    forces the gather kernel on the same data."""
    import torch

    torch.manual_seed(cin * 3 + cout)
    n, h, wd = shape
    x = torch.randn(n, h, wd, cin, device="cuda").bfloat16()
    w = (torch.randn(cout, 9, cin, device="cuda") / (3 * cin ** 0.5)).bfloat16()
    b = torch.randn(cout, device="cuda") * 0.1
    ref = conv_ref(x, w, b, relu=True)
    y_tma = run_conv(gb, x, w, b, True, 0)
    y_gather = run_conv(gb, x, w, b, True, 2)
    e_tma = float((y_tma.float() - ref).norm() / ref.norm())
    e_pair = float((y_tma.float() - y_gather.float()).norm() / ref.norm())
    print("conv tma %d->%d %s: rel err %.2e, tma vs gather %.2e" % (cin, cout, shape, e_tma, e_pair))
    assert e_tma < BF16_TOL
    assert e_pair < 1e-3


@pytest.mark.parametrize("size,batch", [(32, 2), (48, 1), (128, 1)])
def test_unet_exact_case_matches_oracle(gb, size, batch):
    from oracle import unet_ref

    layers, n = unet_ref.layer_table()
    rng = np.random.default_rng(size)
    params = _sparse_params(layers, n, rng)
    x = rng.integers(0, 4, (batch, size, size)).astype(np.float64)
    dout = rng.integers(-1, 2, (batch, size, size)).astype(np.float64)
    e_fwd, errs = _compare(gb, size, batch, params, x, dout)
    worst = max(errs.items(), key=lambda kv: kv[1])
    print("unet exact %dx%d: forward %.1e, worst gradient %s %.1e" % (size, size, e_fwd, *worst))
    assert e_fwd <= EXACT_TOL
    assert worst[1] <= EXACT_GRAD_TOL, errs


@pytest.mark.parametrize("size,batch", [(32, 2), (48, 1)])
def test_unet_random_case_near_oracle(gb, size, batch):
    from oracle import unet_ref

    layers, n = unet_ref.layer_table()
    rng = np.random.default_rng(size + 7)
    params = _random_params(layers, n, rng)
    yy, xx = np.mgrid[0:size, 0:size] / size
    x = np.stack([np.sin(6 * xx + rng.uniform(0, 6)) * np.cos(5 * yy) +
                  0.3 * rng.standard_normal((size, size)) for _ in range(batch)])
    x = x.astype(np.float32).astype(np.float64)
    dout = rng.standard_normal(x.shape).astype(np.float32).astype(np.float64)
    e_fwd, errs = _compare(gb, size, batch, params, x, dout)
    worst = max(errs.items(), key=lambda kv: kv[1])
    print("unet random %dx%d: forward %.2e, worst gradient %s %.2e, median %.2e" %
          (size, size, e_fwd, *worst, float(np.median(list(errs.values())))))
    assert e_fwd < RAND_FWD_TOL
    assert worst[1] < RAND_GRAD_TOL, errs


def _inputs(rng, n, size):
    yy, xx = np.mgrid[0:size, 0:size] / size
    x = np.stack([np.sin(6 * xx + rng.uniform(0, 6)) * np.cos(5 * yy) +
                  0.3 * rng.standard_normal((size, size)) for _ in range(n)])
    return x.astype(np.float32)


def test_unet_train_step_reduces_loss(gb):
    import torch

    size, batch = 64, 4
    net = gb.UNet(size, batch, train=True, seed=5)
    rng = np.random.default_rng(5)
    x = _inputs(rng, batch, size)
    target = x + 0.5 * np.roll(x, 1, axis=2)  # a fixed linear map the net can learn
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(target.astype(np.float32)).cuda()
    losses = [net.train_step(xd, td, 2e-3) for _ in range(60)]
    print("unet training loss %.4e -> %.4e" % (losses[0], losses[-1]))
    assert losses[-1] < 0.2 * losses[0]


def test_multiscale_loss_against_oracle(gb):
    """The multi-scale training loss (error pooled over 2^s blocks, weight
    ratio^s): the loss the library reports matches the oracle's formula on the
    network's own output, and the gradient it trains with agrees with the
    oracle's d loss / d out pushed through the (separately checked) backward
    kernels: on AdamW's first steps every parameter moves against the sign of
    its gradient."""
    import torch

    from oracle import unet_ref

    size, batch, levels, ratio = 64, 2, 4, 2.0
    net = gb.UNet(size, batch, train=True, seed=9)
    net.set_loss(levels, ratio)
    rng = np.random.default_rng(9)
    x = _inputs(rng, batch, size)
    target = (x + 0.3 * np.roll(x, 2, axis=1) + 0.2).astype(np.float32)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(target).cuda()
    y = torch.zeros_like(xd)
    net.forward(xd, y)
    loss_ref, dout = unet_ref.multiscale_loss_grad(y.cpu().numpy(), target, levels, ratio)
    p0 = torch.zeros(net.nparams, device="cuda")
    net.get_params(p0)
    loss = net.train_step(xd, td, 0.0)  # lr 0: the parameters stay
    assert loss == pytest.approx(loss_ref, rel=1e-5)
    g = torch.zeros(net.nparams, device="cuda")
    net.forward(xd, y)
    net.backward(torch.from_numpy(dout.astype(np.float32)).cuda(), g)
    net.train_step(xd, td, 1e-4)
    p1 = torch.zeros_like(p0)
    net.get_params(p1)
    g, step = g.cpu().numpy(), (p1 - p0).cpu().numpy()
    big = np.abs(g) > 1e-3 * np.abs(g).max()
    agree = np.mean(np.sign(step[big]) == -np.sign(g[big]))
    print("multi-scale loss %.6e (oracle %.6e); update direction agrees on %.4f of %d params"
          % (loss, loss_ref, agree, int(big.sum())))
    assert agree > 0.999


@pytest.mark.parametrize("radius,ny,npad", [(31.5, 5, 64), (20.0, 3, 48), (63.5, 9, 128)])
def test_device_images_match_image_cyl2cb(gb, radius, ny, npad):
    """The warm start's device conversion between the cylinder [ray][slice] and
    the network's images [slice][iz][ix] (arecgb_unet_images_from_volume /
    _to_volume) is ImageCyl2CB / ImageCB2Cyl (AREC3D/AREC3D/arecImage.cpp:
    88-232) of the reference-compatible host layer, cube [iz][y][ix] ->
    image y, zero-padded to npad and scaled."""
    import torch

    from conftest import uniform_angles
    from devutil import empty_vol, vol_to_dev

    L = gb.lib()
    plan = gb.Plan(gb.SQ, radius, ny, uniform_angles(4))
    cyl = gb.arecAllocateCylImage(radius, ny)
    assert (cyl.nrays, cyl.nx) == (plan.nrays, plan.nx)
    rng = np.random.default_rng(int(radius))
    x = rng.standard_normal((plan.nrays, ny)).astype(np.float32)
    gb.cyl_data(cyl)[:] = x
    cube = np.zeros((cyl.nz, cyl.ny, cyl.nx), np.float32)
    assert L.arecgb_ImageCyl2CB(cyl, gb._cb_image(cube), cyl.nx, cyl.ny, cyl.nz) == 0
    scale = 0.5
    img = torch.full((ny, npad, npad), 7.0, device="cuda")
    gb.images_from_volume(plan, vol_to_dev(plan, x), img, npad, 0, ny, scale)
    imh = img.cpu().numpy()
    nx = plan.nx
    np.testing.assert_array_equal(imh[:, :nx, :nx], scale * cube.transpose(1, 0, 2))
    assert not imh[:, nx:, :].any() and not imh[:, :, nx:].any()
    # and back: the images of the disk give the cylinder (ImageCB2Cyl)
    back = empty_vol(plan)
    gb.images_to_volume(plan, img, back, npad, 0, ny, 1.0 / scale)
    np.testing.assert_array_equal(back[:, :ny].cpu().numpy(), x)
    gb.arecImageFree(cyl)
    plan.close()
