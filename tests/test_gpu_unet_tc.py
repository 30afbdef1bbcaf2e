"""The network's 3x3 convolutions on the tcgen05 tensor cores (TMEM
accumulators) against a float64 reference computed from the same BF16
operands, against the mma.sync kernels, and with TMA-staged against
thread-staged input rows, through the C-ABI scf_unet_conv.  Every variant the network launches: forward with ReLU,
forward with nearest upsampling and the skip add, and the input gradient
with and without the ReLU mask; shapes with ragged 128-pixel segments,
rows narrower than a segment and several segments per row."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FWD_RELU = [(16, 16), (16, 32), (32, 32), (32, 64), (64, 64)]
FWD_UP = [(64, 64), (64, 32), (32, 16)]
BWD_MASK = [(16, 16), (32, 16), (32, 32), (64, 32), (64, 64)]
BWD_PLAIN = [(64, 64), (32, 64), (16, 32)]
VARIANTS = ([("relu", c) for c in FWD_RELU] + [("up", c) for c in FWD_UP] +
            [("bwd_mask", c) for c in BWD_MASK] + [("bwd", c) for c in BWD_PLAIN])


def _bf16(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(torch.bfloat16)


def _f64(torch, t):
    return t.float().cpu().numpy().astype(np.float64)


def _conv_ref(x, w, n, H, W):
    """x [n][H][W][cin] (float64), w [cout][9][cin] -> [n][H][W][cout]."""
    xp = np.zeros((n, H + 2, W + 2, x.shape[-1]))
    xp[:, 1:H + 1, 1:W + 1] = x
    out = np.zeros((n, H, W, w.shape[0]))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        out += np.einsum("nhwc,oc->nhwo", xp[:, dy:dy + H, dx:dx + W], w[:, tap])
    return out


def _run(torch, engine, kind, cin, cout, n, H, W, seed):
    from simcoflow_gb300 import learned as Lr
    rng = np.random.Generator(np.random.PCG64(seed))
    dev = torch.device("cuda:0")
    ups, bwd, mask = kind == "up", kind.startswith("bwd"), kind == "bwd_mask"
    Hi, Wi = (H // 2, W // 2) if ups else (H, W)
    x = _bf16(torch, rng.normal(size=(n, Hi, Wi, cin))).to(dev)
    w = _bf16(torch, rng.normal(size=(cout, 9, cin)) / np.sqrt(9 * cin)).to(dev)
    b = torch.from_numpy(rng.uniform(-0.5, 0.5, cout).astype(np.float32)).to(dev)
    m = _bf16(torch, rng.normal(size=(n, H, W, cin))).to(dev) if mask else None
    a = _bf16(torch, rng.normal(size=(n, H, W, cout))).to(dev) if ups else None
    out = torch.full((n, H, W, cout), float("nan"), dtype=torch.bfloat16, device=dev)
    ptr = lambda t: C.c_void_p(t.data_ptr() if t is not None else 0)
    rc = Lr.lib().scf_unet_conv(engine, cin, cout, int(ups), int(bwd), int(mask), ptr(x), ptr(m),
                                ptr(w), ptr(None if bwd else b), ptr(a), ptr(out), n, H, W, None)
    assert rc == 0, f"scf_unet_conv returned {rc}"
    torch.cuda.synchronize()
    # reference from the same BF16 operands, float64 sums
    xr = _f64(torch, x)
    if ups:
        xr = xr.repeat(2, axis=1).repeat(2, axis=2)
    if mask:
        xr = np.where(_f64(torch, m) > 0, xr, 0.0)
    ref = _conv_ref(xr, _f64(torch, w), n, H, W)
    if not bwd:
        ref += _f64(torch, b)
    if ups:
        ref += _f64(torch, a)
    if kind == "relu":
        ref = np.maximum(ref, 0.0)
    return _f64(torch, out), ref


def _check(got, ref):
    assert np.isfinite(got).all(), "output pixels not written"
    # one BF16 rounding of the output (relative 2^-8) plus FP32 summation order
    err = np.abs(got - ref)
    assert np.all(err <= 2.0 ** -8 * np.abs(ref) + 1e-3 * (np.abs(ref).max() + 1e-30)), \
        f"max error {err.max():.3e} at {np.unravel_index(err.argmax(), err.shape)}"


@pytest.mark.parametrize("kind,ch", VARIANTS, ids=[f"{k}-{c[0]}x{c[1]}" for k, c in VARIANTS])
def test_tcgen05_conv_matches_reference(cuda, kind, ch):
    import torch
    cin, cout = ch
    # rows narrower than a tile, a ragged second segment, two images
    for (n, H, W) in [(2, 6, 40), (1, 6 if kind == "up" else 5, 136)]:
        got, ref = _run(torch, 1, kind, cin, cout, n, H, W, seed=cin * 7 + cout)
        _check(got, ref)


@pytest.mark.parametrize("kind,ch", [("relu", (64, 64)), ("up", (64, 32)), ("bwd_mask", (32, 16)),
                                     ("relu", (16, 16))])
def test_tcgen05_conv_matches_mma_sync_kernel(cuda, kind, ch):
    import torch
    cin, cout = ch
    n, H, W = 2, 34, 256  # two full segments per row, several rows per CTA strip
    g1, ref = _run(torch, 1, kind, cin, cout, n, H, W, seed=5)
    g0, _ = _run(torch, 0, kind, cin, cout, n, H, W, seed=5)
    _check(g1, ref)
    _check(g0, ref)
    # both accumulate in FP32 from the same BF16 operands: after the BF16
    # rounding of the output they differ by at most one unit in the last place
    d = np.abs(g1 - g0)
    assert np.all(d <= 2.0 ** -7 * np.maximum(np.abs(g0), np.abs(g1)) + 1e-4 * np.abs(g0).max())


FWD_ALL = [("relu", c) for c in FWD_RELU] + [("up", c) for c in FWD_UP]


@pytest.mark.parametrize("kind,ch", FWD_ALL, ids=[f"{k}-{c[0]}x{c[1]}" for k, c in FWD_ALL])
def test_tma_staged_rows_match_thread_staged_rows(cuda, kind, ch):
    """Engine 1 stages the forward layers' input rows by TMA (an upsampling
    layer copies the half-resolution row and expands it in shared memory),
    engine 2 with the CTA's threads: the same MMAs on the same shared-memory
    layout, so the outputs agree bit for bit (rows of 40, 136 and 256
    pixels, a column of images taller than a tile strip)."""
    import torch
    cin, cout = ch
    for (n, H, W) in [(2, 6, 40), (1, 6 if kind == "up" else 5, 136), (2, 34, 256)]:
        g1, ref = _run(torch, 1, kind, cin, cout, n, H, W, seed=cin + cout)
        g2, _ = _run(torch, 2, kind, cin, cout, n, H, W, seed=cin + cout)
        _check(g1, ref)
        assert np.array_equal(g1, g2)


def test_network_forward_same_on_both_engines(cuda):
    from simcoflow_gb300 import learned as Lr
    rng = np.random.Generator(np.random.PCG64(2))
    n, H, W = 2, 64, 136
    x5 = rng.normal(size=(n, H, W, 5)).astype(np.float32)
    p = Lr.init_params(4)
    net = Lr.UNet(n, H, W)
    try:
        net.set_params(p)
        net.set_input(x5)
        z1 = net.forward()
        net.set_engine(2)
        z2 = net.forward()
        net.set_engine(0)
        z0 = net.forward()
    finally:
        net.close()
    assert np.isfinite(z1).all()
    assert np.array_equal(z1, z2)  # TMA or thread staging: the same MMAs
    assert np.linalg.norm(z1 - z0) <= 2e-2 * np.linalg.norm(z0)
