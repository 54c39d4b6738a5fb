"""CPU restatement of the learned denoiser (test infrastructure only).

This is the checker for the GPU denoiser kernels: the U-Net's forward pass,
its L1 loss and the gradients of every parameter, written with numpy from
the network's mathematical definition. The reference renderer has no
denoiser, so there is nothing of the reference to pin this to: parity with
it is unpinned, and the restatement is pinned instead by a finite-difference
check of its own gradients (tests/test_denoise_oracle.py).

Where the GPU rounds to bf16 (weights, every stored activation and
gradient tensor) this restatement rounds at the same places, so GPU and
restatement differ only by the order of fp32 sums and the bf16 roundings
those can flip. Layouts follow the C ABI: images NHWC, weights
[cout][3][3][cin] (tap 3 (dy + 1) + (dx + 1)), parameters per layer weights
then bias.
"""
import numpy as np

# (cin, cout) of the 15 convolutions in execution order
LAYERS = [(16, 32), (32, 32), (32, 64), (64, 64), (64, 128), (128, 128), (128, 256), (256, 256),
          (384, 128), (128, 128), (192, 64), (64, 64), (96, 32), (32, 32), (32, 16)]
IN_C, OUT_C, COLOR_C = 16, 16, 3


def bf16(x):
    """Round float32 to the nearest bfloat16 (ties to even), as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    nan = np.isnan(x)
    if nan.any():
        out = np.where(nan, x, out)
    return out.reshape(x.shape)


def unpack(params):
    """Per layer (W [cout,3,3,cin], b [cout]) views of the flat parameter array."""
    out, off = [], 0
    for cin, cout in LAYERS:
        n = cout * 9 * cin
        w = params[off:off + n].reshape(cout, 3, 3, cin)
        off += n
        b = params[off:off + cout]
        off += cout
        out.append((w, b))
    assert off == len(params)
    return out


def num_params():
    return sum(cout * 9 * cin + cout for cin, cout in LAYERS)


def im2col(x):
    """(N,H,W,C) -> (N*H*W, 9*C), tap-major, zero padding."""
    N, H, W, C = x.shape
    xp = np.zeros((N, H + 2, W + 2, C), np.float32)
    xp[:, 1:-1, 1:-1] = x
    cols = [xp[:, dy:dy + H, dx:dx + W] for dy in range(3) for dx in range(3)]
    return np.concatenate(cols, axis=-1).reshape(N * H * W, 9 * C)


def conv(x, w, b=None):
    """3x3 convolution, fp32 sums of (bf16) operands."""
    N, H, W, C = x.shape
    cout = w.shape[0]
    y = im2col(x) @ w.reshape(cout, 9 * C).T.astype(np.float32)
    if b is not None:
        y = y + b[None, :]
    return y.reshape(N, H, W, cout).astype(np.float32)


def conv_input_grad(dy, w):
    """Gradient of conv() with respect to its input: the convolution of dy with
    the spatially flipped, channel-transposed weights."""
    wt = np.transpose(w[:, ::-1, ::-1, :], (3, 1, 2, 0))  # [cin][3][3][cout]
    return conv(dy, np.ascontiguousarray(wt))


def conv_weight_grad(dy, x):
    N, H, W, C = x.shape
    cout = dy.shape[-1]
    g = dy.reshape(-1, cout).T @ im2col(x)  # (cout, 9*C)
    return g.reshape(cout, 3, 3, C)


def maxpool(x):
    N, H, W, C = x.shape
    v = x.reshape(N, H // 2, 2, W // 2, 2, C)
    return v.max(axis=(2, 4))


def maxpool_grad(x, dy):
    """To the first maximum of each window in the order (0,0), (0,1), (1,0), (1,1)."""
    N, H, W, C = x.shape
    v = x.reshape(N, H // 2, 2, W // 2, 2, C).transpose(0, 1, 3, 2, 4, 5).reshape(N, H // 2, W // 2, 4, C)
    arg = v.argmax(axis=3)  # first occurrence of the maximum
    onehot = (np.arange(4)[None, None, None, :, None] == arg[:, :, :, None, :])
    g = (onehot * dy[:, :, :, None, :]).astype(np.float32)
    g = g.reshape(N, H // 2, W // 2, 2, 2, C).transpose(0, 1, 3, 2, 4, 5).reshape(N, H, W, C)
    return g


def upsample(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def upsample_grad(dy):
    N, H, W, C = dy.shape
    return dy.reshape(N, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4), dtype=np.float32)


def relu(x):
    return np.maximum(x, 0.0).astype(np.float32)


def forward(params, x):
    """Activations of every layer (bf16-rounded as the GPU stores them) and
    the fp32 output (N,H,W,16)."""
    L = unpack(params)
    Wb = [(bf16(w), b) for w, b in L]
    a = {}

    def c(i, inp, act=True):
        w, b = Wb[i]
        y = conv(inp, w, b)
        return bf16(relu(y)) if act else y

    a["x"] = bf16(x)
    a["a0"] = c(0, a["x"]);      a["e0"] = c(1, a["a0"]);  a["p0"] = maxpool(a["e0"])
    a["a1"] = c(2, a["p0"]);     a["e1"] = c(3, a["a1"]);  a["p1"] = maxpool(a["e1"])
    a["a2"] = c(4, a["p1"]);     a["e2"] = c(5, a["a2"]);  a["p2"] = maxpool(a["e2"])
    a["a3"] = c(6, a["p2"]);     a["e3"] = c(7, a["a3"])
    a["cat2"] = np.concatenate([upsample(a["e3"]), a["e2"]], -1)
    a["b2"] = c(8, a["cat2"]);   a["d2"] = c(9, a["b2"])
    a["cat1"] = np.concatenate([upsample(a["d2"]), a["e1"]], -1)
    a["b1"] = c(10, a["cat1"]);  a["d1"] = c(11, a["b1"])
    a["cat0"] = np.concatenate([upsample(a["d1"]), a["e0"]], -1)
    a["b0"] = c(12, a["cat0"]);  a["d0"] = c(13, a["b0"])
    a["out"] = c(14, a["d0"], act=False)
    a["out"][..., :COLOR_C] += a["x"][..., :COLOR_C]  # residual on the input's log colour
    return a


def loss_and_grads(params, x, target):
    """L1 loss of the first 3 output channels against log(1 + target) and the
    gradient of every parameter (flat fp32 array, the C ABI's order)."""
    L = unpack(params)
    Wb = [bf16(w) for w, _ in L]
    a = forward(params, x)
    out = a["out"]
    t = np.log1p(np.maximum(target[..., :COLOR_C], 0.0)).astype(np.float32)
    d = out[..., :COLOR_C] - t
    n = d.size
    loss = float(np.abs(d).sum(dtype=np.float64) / n)
    gout = np.zeros(out.shape, np.float32)
    gout[..., :COLOR_C] = np.sign(d) / np.float32(n)
    gout = bf16(gout)
    gW = [None] * len(LAYERS)
    gb = [None] * len(LAYERS)

    def back(i, inp, dy, mask):
        gW[i] = conv_weight_grad(dy, inp)
        gb[i] = dy.reshape(-1, dy.shape[-1]).sum(axis=0, dtype=np.float32)
        if mask is None:
            return None
        dx = conv_input_grad(dy, Wb[i])
        return bf16(np.where(mask > 0, dx, 0.0).astype(np.float32))

    g = {}
    g["d0"] = back(14, a["d0"], gout, a["d0"])
    g["b0"] = back(13, a["b0"], g["d0"], a["b0"])
    g["cat0"] = back(12, a["cat0"], g["b0"], a["cat0"])
    g["d1"] = bf16(upsample_grad(g["cat0"][..., :64]))
    g["b1"] = back(11, a["b1"], g["d1"], a["b1"])
    g["cat1"] = back(10, a["cat1"], g["b1"], a["cat1"])
    g["d2"] = bf16(upsample_grad(g["cat1"][..., :128]))
    g["b2"] = back(9, a["b2"], g["d2"], a["b2"])
    g["cat2"] = back(8, a["cat2"], g["b2"], a["cat2"])
    g["e3"] = bf16(upsample_grad(g["cat2"][..., :256]))
    g["a3"] = back(7, a["a3"], g["e3"], a["a3"])
    g["p2"] = back(6, a["p2"], g["a3"], a["p2"])
    g["e2"] = bf16(maxpool_grad(a["e2"], g["p2"]) + g["cat2"][..., 256:])
    g["a2"] = back(5, a["a2"], g["e2"], a["a2"])
    g["p1"] = back(4, a["p1"], g["a2"], a["p1"])
    g["e1"] = bf16(maxpool_grad(a["e1"], g["p1"]) + g["cat1"][..., 128:])
    g["a1"] = back(3, a["a1"], g["e1"], a["a1"])
    g["p0"] = back(2, a["p0"], g["a1"], a["p0"])
    g["e0"] = bf16(maxpool_grad(a["e0"], g["p0"]) + g["cat0"][..., 64:])
    g["a0"] = back(1, a["a0"], g["e0"], a["a0"])
    back(0, a["x"], g["a0"], None)
    flat = np.concatenate([np.concatenate([gW[i].reshape(-1), gb[i]]) for i in range(len(LAYERS))])
    return loss, flat.astype(np.float32), a


def exact_loss(params, x, target):
    """The loss in float64 without any bf16 rounding (for finite differences)."""
    L = unpack(params)
    h = x.astype(np.float64)

    def c(i, inp, act=True):
        w, b = L[i]
        N, H, W, C = inp.shape
        xp = np.zeros((N, H + 2, W + 2, C))
        xp[:, 1:-1, 1:-1] = inp
        cols = np.concatenate([xp[:, dy:dy + H, dx:dx + W] for dy in range(3) for dx in range(3)], -1)
        y = cols.reshape(N * H * W, 9 * C) @ w.reshape(w.shape[0], 9 * C).T.astype(np.float64) + b
        y = y.reshape(N, H, W, -1)
        return np.maximum(y, 0.0) if act else y

    def mp(v):
        N, H, W, C = v.shape
        return v.reshape(N, H // 2, 2, W // 2, 2, C).max(axis=(2, 4))

    def up(v):
        return np.repeat(np.repeat(v, 2, 1), 2, 2)

    a0 = c(0, h); e0 = c(1, a0); a1 = c(2, mp(e0)); e1 = c(3, a1); a2 = c(4, mp(e1)); e2 = c(5, a2)
    a3 = c(6, mp(e2)); e3 = c(7, a3)
    d2 = c(9, c(8, np.concatenate([up(e3), e2], -1)))
    d1 = c(11, c(10, np.concatenate([up(d2), e1], -1)))
    d0 = c(13, c(12, np.concatenate([up(d1), e0], -1)))
    out = c(14, d0, act=False)
    out[..., :COLOR_C] += h[..., :COLOR_C]
    t = np.log1p(np.maximum(target[..., :COLOR_C].astype(np.float64), 0.0))
    return float(np.abs(out[..., :COLOR_C] - t).mean())


def init_params(seed):
    """He-normal weights, zero biases, output channels 3..15 zero. (The GPU's
    own initialisation also zeroes the output layer's colour channels; tests
    use this one so that every layer's gradient is non-zero.)"""
    rng = np.random.default_rng(seed)
    parts = []
    for i, (cin, cout) in enumerate(LAYERS):
        w = rng.normal(0.0, np.sqrt(2.0 / (9 * cin)), (cout, 3, 3, cin)).astype(np.float32)
        if i == len(LAYERS) - 1:
            w[COLOR_C:] = 0.0
        parts += [w.reshape(-1), np.zeros(cout, np.float32)]
    return np.concatenate(parts)
