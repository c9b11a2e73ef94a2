"""CPU oracle of the learned-warm-start U-Net (test infrastructure only).

The reference has no network; this module restates the GPU library's own
architecture (arec3d_gb300/csrc/arec_unet.cu) in PyTorch FP64 on the CPU so
the hand-written forward and backward kernels can be checked against autograd.
With ``bf16=True`` it rounds at the points where the GPU path stores bf16: the
weights of the tensor-core layers and every post-ReLU activation.  The first
layer (1 -> 32) and the 1x1 output layer use FP32 weights on the GPU and are
not rounded here either.

Parameter layout (flat vector, per layer W then b):
  3x3 layers W [Cout][9][Cin], tap t = 3*(dy+1) + (dx+1);  output W [Cin].
"""
import numpy as np

LAYERS = ("c1a", "c1b", "c2a", "c2b", "c3a", "c3b", "c4a", "c4b", "u3", "d3a", "d3b",
          "u2", "d2a", "d2b", "u1", "d1a", "d1b", "out")


CIN = (1, 32, 32, 64, 64, 128, 128, 256, 256, 256, 128, 128, 128, 64, 64, 64, 32, 32)
COUT = (32, 32, 64, 64, 128, 128, 256, 256, 128, 128, 128, 64, 64, 64, 32, 32, 32, 1)


def layer_table():
    """Layer offsets in the flat parameter vector (each block padded to a
    multiple of 8 floats) and the total length."""
    layers, off = [], 0
    for name, ci, co in zip(LAYERS, CIN, COUT):
        nw = ci if name == "out" else co * 9 * ci
        w_off = off
        off += nw
        b_off = off
        off += (co + 7) // 8 * 8
        layers.append(dict(name=name, w_off=w_off, b_off=b_off, cin=ci, cout=co))
    return layers, off


def _rounding_functions():
    """(value rounding with the gradient passed through, identity with the
    gradient rounded): bf16 round-to-nearest-even both."""
    import torch

    class RoundValue(torch.autograd.Function):
        @staticmethod
        def forward(ctx, t):
            return t.to(torch.bfloat16).to(t.dtype)

        @staticmethod
        def backward(ctx, g):
            return g

    class RoundGrad(torch.autograd.Function):
        @staticmethod
        def forward(ctx, t):
            return t.clone()

        @staticmethod
        def backward(ctx, g):
            return g.to(torch.bfloat16).to(g.dtype)

    return RoundValue.apply, RoundGrad.apply


def unpack(params, layers, requires_grad=False):
    """Flat FP32 vector -> {name: (W [Cout, Cin, 3, 3] or [Cin], b [Cout])} in FP64."""
    import torch

    p = torch.as_tensor(np.asarray(params, np.float64))
    out = {}
    for l in layers:
        ci, co = l["cin"], l["cout"]
        if l["name"] == "out":
            w = p[l["w_off"]:l["w_off"] + ci].clone()
        else:
            w = p[l["w_off"]:l["w_off"] + co * 9 * ci].reshape(co, 3, 3, ci).permute(0, 3, 1, 2)
            w = w.contiguous()
        b = p[l["b_off"]:l["b_off"] + co].clone()
        w.requires_grad_(requires_grad)
        b.requires_grad_(requires_grad)
        out[l["name"]] = (w, b)
    return out


def pack_grads(tensors, layers, nparams):
    """Inverse of unpack for the gradients (FP64 numpy, padding zero)."""
    g = np.zeros(nparams)
    for l in layers:
        w, b = tensors[l["name"]]
        gw = w.grad.detach()
        if l["name"] != "out":
            gw = gw.permute(0, 2, 3, 1)  # [Cout, 3, 3, Cin]
        gw = gw.reshape(-1).numpy()
        g[l["w_off"]:l["w_off"] + gw.size] = gw
        g[l["b_off"]:l["b_off"] + l["cout"]] = b.grad.detach().numpy()
    return g


def forward(t, x, bf16=True):
    """t: unpack()ed tensors; x: [N, H, W] tensor -> [N, H, W].

    With bf16, values are rounded where the GPU stores bf16 (tensor-core
    weights, every post-ReLU activation) and gradients where the GPU stores
    bf16 gradients: the input of every tensor-core convolution (its data
    gradient), the skip tensors e1..e3 (pool + skip gradients summed, then
    rounded), the inputs of the upsamplings and of the output layer."""
    import torch
    import torch.nn.functional as F

    if bf16:
        rv, rg = _rounding_functions()
    else:
        rv = rg = (lambda v: v)

    def conv(name, h, tensor_core=True):
        w, b = t[name]
        if tensor_core:
            w, h = rv(w), rg(h)
        return rv(torch.relu(F.conv2d(h, w, b, padding=1)))

    def up(h):
        return F.interpolate(rg(h), scale_factor=2, mode="nearest")

    a1 = conv("c1a", x[:, None], tensor_core=False)
    e1 = rg(conv("c1b", a1))
    e2 = rg(conv("c2b", conv("c2a", F.max_pool2d(e1, 2))))
    e3 = rg(conv("c3b", conv("c3a", F.max_pool2d(e2, 2))))
    e4 = conv("c4b", conv("c4a", F.max_pool2d(e3, 2)))
    g3 = conv("d3b", conv("d3a", torch.cat([conv("u3", up(e4)), e3], 1)))
    g2 = conv("d2b", conv("d2a", torch.cat([conv("u2", up(g3)), e2], 1)))
    g1 = conv("d1b", conv("d1a", torch.cat([conv("u1", up(g2)), e1], 1)))
    w, b = t["out"]
    return (rg(g1) * w[None, :, None, None]).sum(1) + b[0] + x


def forward_and_grads(params, layers, nparams, x, dout, bf16=True):
    """Output and d(sum(out * dout))/d(params) as FP64 numpy arrays."""
    import torch

    t = unpack(params, layers, requires_grad=True)
    xt = torch.as_tensor(np.asarray(x, np.float64))
    y = forward(t, xt, bf16=bf16)
    (y * torch.as_tensor(np.asarray(dout, np.float64))).sum().backward()
    return y.detach().numpy(), pack_grads(t, layers, nparams)


def multiscale_loss_grad(out, target, levels, ratio):
    """The library's multi-scale training loss and its gradient w.r.t. the
    output, in FP64: with e = out - target and level s the error averaged over
    2^s x 2^s blocks (level 0 = e), loss = sum_s ratio^s * mean(level_s^2) and
    d loss / d out(p) = 2 / P * sum_s ratio^s * level_s(block of p), P the
    number of pixels (the mean over level s is over P / 4^s cells, each holding
    4^s pixels).  out, target: [N][H][W]."""
    e = np.asarray(out, np.float64) - np.asarray(target, np.float64)
    n, h, w = e.shape
    P = e.size
    loss = float(np.mean(e * e))
    grad = e.copy()
    lev = e
    for s in range(1, levels + 1):
        lev = 0.25 * (lev[:, 0::2, 0::2] + lev[:, 1::2, 0::2] + lev[:, 0::2, 1::2] +
                      lev[:, 1::2, 1::2])
        a = float(ratio) ** s
        loss += a * float(np.mean(lev * lev))
        grad += a * np.repeat(np.repeat(lev, 2 ** s, axis=1), 2 ** s, axis=2)
    return loss, 2.0 / P * grad
