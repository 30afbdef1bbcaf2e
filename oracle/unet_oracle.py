"""CPU oracle of the learned preconditioner's network (test infrastructure).

A numpy restatement of the U-Net declared in include/scf_unet.h -- forward
pass, loss and the backward pass to every parameter -- used to check the
CUDA kernels' outputs and gradients.  It rounds to BF16 exactly where the
CUDA path stores BF16 (weights, activations, activation gradients) and
accumulates in FP32, so the two agree up to FP32 summation order and the
BF16 roundings that order can flip.  The network has no reference
counterpart (the reference preconditions with BoomerAMG,
src/ProjectionP_Mod.f90:101-135); nothing here is shipped or measured.
"""
import numpy as np

# cin, cout, level, ups, relu, skip (see include/scf_unet.h)
LAYERS = [(16, 16, 0, False, True, -1), (16, 16, 0, False, True, -1),
          (16, 32, 1, False, True, -1), (32, 32, 1, False, True, -1),
          (32, 64, 2, False, True, -1), (64, 64, 2, False, True, -1),
          (64, 64, 3, False, True, -1), (64, 64, 3, False, True, -1),
          (64, 64, 2, True, False, 5), (64, 64, 2, False, True, -1),
          (64, 32, 1, True, False, 3), (32, 32, 1, False, True, -1),
          (32, 16, 0, True, False, 1), (16, 16, 0, False, True, -1)]


def offsets():
    """(W offset, bias offset) of every layer, and the total parameter count."""
    offs, o = [], 0
    for cin, cout, *_ in LAYERS:
        w = o
        o += cout * 9 * cin
        offs.append((w, o))
        o += cout
    return offs, o + 17


def num_params():
    return offsets()[1]


def bf16(x):
    """Round float32 to the nearest BF16 value (ties to even), as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(x.shape)


def init_params(seed=0):
    """He-uniform weights, zero biases, small head; float32."""
    rng = np.random.Generator(np.random.PCG64(seed))
    offs, n = offsets()
    p = np.zeros(n, np.float32)
    for (cin, cout, *_), (wo, bo) in zip(LAYERS, offs):
        a = np.sqrt(6.0 / (9 * (5 if wo == 0 else cin)))
        p[wo:bo] = rng.uniform(-a, a, cout * 9 * cin)
    p[n - 17:n - 1] = rng.uniform(-0.25, 0.25, 16)
    return p


def _weights(p, i):
    offs, _ = offsets()
    cin, cout = LAYERS[i][:2]
    wo, bo = offs[i]
    return bf16(p[wo:bo].reshape(cout, 9, cin)), p[bo:bo + cout].astype(np.float32)


def _conv(x, w, up=False):
    """3x3 'same' correlation of NHWC x with w [cout][9][cin], FP32 sums."""
    if up:
        x = x.repeat(2, axis=1).repeat(2, axis=2)
    n, H, W, _ = x.shape
    xp = np.zeros((n, H + 2, W + 2, x.shape[3]), np.float32)
    xp[:, 1:-1, 1:-1] = x
    out = np.zeros((n, H, W, w.shape[0]), np.float32)
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        out += np.einsum("nhwc,oc->nhwo", xp[:, dy:dy + H, dx:dx + W], w[:, tap, :],
                         dtype=np.float32)
    return out


def _conv_t(g, w):
    """Input gradient of _conv (no upsampling): correlation with flipped,
    transposed weights."""
    wt = w[:, ::-1, :].transpose(2, 1, 0)  # [cin][9][cout]
    return _conv(g, np.ascontiguousarray(wt))


def _pool(x):
    n, H, W, C = x.shape
    return x.reshape(n, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4), dtype=np.float32)


def _sumpool(x):
    n, H, W, C = x.shape
    return x.reshape(n, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4), dtype=np.float32)


def forward(p, x5):
    """x5: [n][H][W][5] input features.  Returns (z [n][H][W], cache)."""
    n, H, W, _ = x5.shape
    xin = np.zeros((n, H, W, 16), np.float32)
    xin[..., :5] = bf16(x5)
    acts, pools = [], {}
    for i, (cin, cout, lev, up, relu, skip) in enumerate(LAYERS):
        if i == 0:
            xi = xin
        elif i in (2, 4, 6):
            xi = bf16(_pool(acts[i - 1]))
            pools[i] = xi
        else:
            xi = acts[i - 1]
        w, b = _weights(p, i)
        y = _conv(xi, w, up) + b
        if skip >= 0:
            y = y + acts[skip]
        if relu:
            y = np.maximum(y, 0.0)
        acts.append(bf16(y))
    hw = p[-17:-1].astype(np.float32)
    z = np.einsum("nhwc,c->nhw", acts[-1], hw, dtype=np.float32) + p[-1]
    return z, {"xin": xin, "acts": acts, "pools": pools}


def loss(z, t, mask):
    """sum over images of sum_mask (z-t)^2 / sum_mask t^2, and dL/dz."""
    m = mask.astype(np.float32)
    tt = (t * t * m).sum(axis=(1, 2))
    se = (((z - t) ** 2) * m).sum(axis=(1, 2))
    L = float(np.sum(np.where(tt > 0, se / np.where(tt > 0, tt, 1), 0.0)))
    sc = np.where(tt > 0, 2.0 / np.where(tt > 0, tt, 1), 0.0)[:, None, None]
    return L, (sc * (z - t) * m).astype(np.float32)


def backward(p, cache, dz):
    """Gradient of sum(dz * z) with respect to every parameter (float32)."""
    offs, n = offsets()
    g = np.zeros(n, np.float32)
    acts, pools, xin = cache["acts"], cache["pools"], cache["xin"]
    hw = p[-17:-1].astype(np.float32)
    g[-17:-1] = np.einsum("nhw,nhwc->c", dz, acts[-1], dtype=np.float32)
    g[-1] = dz.sum(dtype=np.float32)
    gout = bf16(dz[..., None] * hw)  # gradient of d0
    gskip = {}
    for i in range(len(LAYERS) - 1, -1, -1):
        cin, cout, lev, up, relu, skip = LAYERS[i]
        wo, bo = offs[i]
        xi = xin if i == 0 else pools[i] if i in (2, 4, 6) else acts[i - 1]
        dpre = gout * (acts[i] > 0) if relu else gout
        xu = xi.repeat(2, axis=1).repeat(2, axis=2) if up else xi
        nimg, H, W, _ = xu.shape
        xp = np.zeros((nimg, H + 2, W + 2, cin), np.float32)
        xp[:, 1:-1, 1:-1] = xu
        dw = np.zeros((cout, 9, cin), np.float32)
        for tap in range(9):
            dy, dx = divmod(tap, 3)
            dw[:, tap, :] = np.einsum("nhwo,nhwc->oc", dpre, xp[:, dy:dy + H, dx:dx + W],
                                      dtype=np.float32)
        g[wo:bo] = dw.ravel()
        g[bo:bo + cout] = dpre.sum(axis=(0, 1, 2), dtype=np.float32)
        if skip >= 0:
            gskip[skip] = gout
        if i == 0:
            break
        w, _ = _weights(p, i)
        gin = bf16(_conv_t(dpre, w))
        if up:
            gin = bf16(_sumpool(gin))
        if i in (2, 4, 6):
            gin = bf16(gskip[i - 1] + 0.25 * gin.repeat(2, axis=1).repeat(2, axis=2))
        gout = gin
    return g
