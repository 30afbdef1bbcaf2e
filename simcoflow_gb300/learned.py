"""Learned preconditioner: the U-Net of include/scf_unet.h (host side).

* `UNet`            ctypes handle over the scf_unet_* C-ABI (training and tests)
* `init_params`     He-uniform initialisation
* `generate_pairs`  residual/error pairs (r_k, e_k = x* - x_k) of the plain
                    MG-PCG on seeded projection instances (the training set)
* `train`           Adam on the normalised error loss, with the CUDA forward
                    and backward kernels
* `save` / `load_weights`  the weights file shipped with the package

The network has no reference counterpart; the reference preconditions its
PCG with BoomerAMG (src/ProjectionP_Mod.f90:116-133).  Training runs on the
GPU only; there is no CPU path.

Command line (writes the weights file):
    python -m simcoflow_gb300.learned --instances 250 --iters 16 --size 512 \\
        --steps 1500 --batch 8 --out simcoflow_gb300/weights/unet_c4.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import pathlib
import time

import numpy as np

from . import projection as P

WEIGHTS = pathlib.Path(__file__).resolve().parent / "weights" / "unet_c4.npz"

# cin, cout of the 14 convolution layers (include/scf_unet.h)
LAYERS = [(16, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 64), (64, 64),
          (64, 64), (64, 64), (64, 32), (32, 32), (32, 16), (16, 16)]

_bound = False


def lib():
    global _bound
    L = P.load()
    if not _bound:
        vp, ip, fp = C.c_void_p, C.c_int, C.c_float
        L.scf_unet_num_params.argtypes = []
        L.scf_unet_create.argtypes = [C.POINTER(vp), ip, ip, ip, ip]
        L.scf_unet_destroy.argtypes = [vp]
        L.scf_unet_set_stream.argtypes = [vp, vp]
        L.scf_unet_set_params.argtypes = [vp, vp]
        L.scf_unet_get_params.argtypes = [vp, vp]
        L.scf_unet_features.argtypes = [vp, ip, ip, ip, vp, vp, vp, vp, vp]
        L.scf_unet_target.argtypes = [vp, ip, ip, ip, vp, vp, vp, vp, vp]
        L.scf_unet_set_input.argtypes = [vp, vp]
        L.scf_unet_forward.argtypes = [vp, vp, ip]
        L.scf_unet_loss.argtypes = [vp, vp, vp, C.POINTER(fp)]
        L.scf_unet_set_dz.argtypes = [vp, vp]
        L.scf_unet_backward.argtypes = [vp]
        L.scf_unet_get_grads.argtypes = [vp, vp]
        L.scf_unet_adam.argtypes = [vp, fp, fp, fp, fp, ip]
        L.scf_unet_set_engine.argtypes = [vp, ip]
        L.scf_unet_conv.argtypes = [ip, ip, ip, ip, ip, ip, vp, vp, vp, vp, vp, vp, ip, ip, ip,
                                    vp]
        for name in P.UNET_EXPORTS:
            getattr(L, name).restype = C.c_int
        _bound = True
    return L


def num_params() -> int:
    return lib().scf_unet_num_params()


def _ck(rc, where):
    if rc != 0:
        raise RuntimeError(f"{where} failed ({rc})")


class UNet:
    """A batch of n images of h x w cells (multiples of 8) on one GPU."""

    def __init__(self, n: int, h: int, w: int, device: int = 0):
        self.n, self.h, self.w = n, h, w
        hd = C.c_void_p()
        _ck(lib().scf_unet_create(C.byref(hd), n, h, w, device), "scf_unet_create")
        self._h = hd

    def close(self):
        if getattr(self, "_h", None):
            lib().scf_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_engine(self, engine: int):
        """Convolution engine: 1 = tcgen05 (default), 0 = mma.sync (comparison)."""
        _ck(lib().scf_unet_set_engine(self._h, engine), "scf_unet_set_engine")

    def set_stream(self, ptr: int):
        _ck(lib().scf_unet_set_stream(self._h, C.c_void_p(ptr)), "scf_unet_set_stream")

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == num_params()
        _ck(lib().scf_unet_set_params(self._h, p.ctypes.data), "scf_unet_set_params")

    def get_params(self):
        p = np.zeros(num_params(), np.float32)
        _ck(lib().scf_unet_get_params(self._h, p.ctypes.data), "scf_unet_get_params")
        return p

    def features(self, i, nx, ny, r, cE, cN, dg, sigma):
        """r, cE, cN, dg: CUDA float64 tensors (Fortran (nx,ny)); sigma: CUDA float32."""
        _ck(lib().scf_unet_features(self._h, i, nx, ny, r.data_ptr(), cE.data_ptr(), cN.data_ptr(),
                                    dg.data_ptr(), sigma.data_ptr()), "scf_unet_features")

    def target(self, i, nx, ny, e, dg, sigma, t, mask):
        _ck(lib().scf_unet_target(self._h, i, nx, ny, e.data_ptr(), dg.data_ptr(),
                                  sigma.data_ptr(), t.data_ptr(), mask.data_ptr()),
            "scf_unet_target")

    def set_input(self, x5):
        x5 = np.ascontiguousarray(x5, dtype=np.float32)
        assert x5.shape == (self.n, self.h, self.w, 5)
        _ck(lib().scf_unet_set_input(self._h, x5.ctypes.data), "scf_unet_set_input")

    def forward(self, z=None):
        """Returns z (numpy) or writes it into the CUDA tensor z."""
        if z is None:
            out = np.zeros((self.n, self.h, self.w), np.float32)
            _ck(lib().scf_unet_forward(self._h, out.ctypes.data, 0), "scf_unet_forward")
            return out
        _ck(lib().scf_unet_forward(self._h, z.data_ptr(), 1), "scf_unet_forward")
        return z

    def loss(self, t, mask) -> float:
        v = C.c_float(0.0)
        _ck(lib().scf_unet_loss(self._h, t.data_ptr(), mask.data_ptr(), C.byref(v)),
            "scf_unet_loss")
        return float(v.value)

    def set_dz(self, dz):
        dz = np.ascontiguousarray(dz, dtype=np.float32)
        _ck(lib().scf_unet_set_dz(self._h, dz.ctypes.data), "scf_unet_set_dz")

    def backward(self):
        _ck(lib().scf_unet_backward(self._h), "scf_unet_backward")

    def grads(self):
        g = np.zeros(num_params(), np.float32)
        _ck(lib().scf_unet_get_grads(self._h, g.ctypes.data), "scf_unet_get_grads")
        return g

    def adam(self, lr, step, b1=0.9, b2=0.999, eps=1e-8):
        _ck(lib().scf_unet_adam(self._h, lr, b1, b2, eps, step), "scf_unet_adam")


def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform weights (fan-in 9 x input channels; 5 real channels in the
    first layer), zero biases, head weights U(-0.25, 0.25)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(num_params(), np.float32)
    o = 0
    for i, (cin, cout) in enumerate(LAYERS):
        a = np.sqrt(6.0 / (9 * (5 if i == 0 else cin)))
        p[o:o + cout * 9 * cin] = rng.uniform(-a, a, cout * 9 * cin)
        o += cout * 9 * cin + cout
    p[o:o + 16] = rng.uniform(-0.25, 0.25, 16)
    return p


def save(params, path, meta=None):
    path = pathlib.Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, params=np.asarray(params, np.float32),
                        meta=json.dumps(meta or {}))


def load_weights(path=WEIGHTS):
    """(params, meta) of a weights file; raises if it is missing."""
    with np.load(path) as z:
        return z["params"].astype(np.float32), json.loads(str(z["meta"]))


def _device_case(case, dev):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).to(dev)
            for k, v in case.arrays.items() if isinstance(v, np.ndarray)}


def generate_pairs(n_inst=250, n_iter=16, size=512, config=4, seed=None, device=0, log=None):
    """Training pairs of the plain FP64 MG-PCG: for each seeded instance
    (0-4 circles, sinusoidal interface, log-uniform density ratio), the
    projection right-hand side b, x* to rtol 1e-12, and for k < n_iter the
    iterate x_k (k PCG iterations) with r_k = b - A x_k and e_k = x* - x_k.
    Returns dict of CUDA tensors: ops [n_inst][3][nx*ny] (cE, cN, dg), r, e
    [n_inst*n_iter][nx*ny], inst index per pair."""
    import torch
    from gen import synth
    dev = torch.device("cuda", device)
    nn = size * size
    ops = torch.zeros((n_inst, 3, nn), dtype=torch.float64, device=dev)
    R = torch.zeros((n_inst * n_iter, nn), dtype=torch.float64, device=dev)
    E = torch.zeros_like(R)
    inst = np.repeat(np.arange(n_inst), n_iter)
    t0 = time.time()
    for i in range(n_inst):
        c = synth.random_instance(config, size, i, seed=seed)
        t = _device_case(c, dev)
        s = P.ProjectionSolver(size, size, precision="fp64", device_ptrs=True, rtol=1e-12,
                               maxit=300)
        try:
            s.set_grid(t["dx"], t["dy"], t["dxU"], t["dyV"])
            s.set_geometry(**{k: t[k] for k in P.GEOMETRY_ARGS})
            s.assemble(t["DpU"], t["DpV"], c.betaP, c.betaM, c.bc)
            # one projection fills the right-hand side b of the instance
            Pp = torch.zeros_like(t["p0"])
            mres = torch.zeros(nn, dtype=torch.float64, device=dev)
            s.update_puv(t["ustar"], t["vstar"], t["u0"].clone(), t["v0"].clone(),
                         t["p0"].clone(), c.vb, Pp=Pp, mres=mres)
            op = s.get_operator()
            for j, k in enumerate(("cE", "cN", "diag")):
                ops[i, j] = torch.from_numpy(np.ascontiguousarray(op[k].ravel(order="F"))).to(dev)
            b = torch.from_numpy(np.ascontiguousarray(op["rhs"].ravel(order="F"))).to(dev)
            xs, _, _ = s.solve_rhs(b)
            for k in range(n_iter):
                xk, rk, _ = s.solve_rhs(b, maxit=k, check=False)
                R[i * n_iter + k] = rk
                E[i * n_iter + k] = xs - xk
        finally:
            s.close()
        if log and (i + 1) % 25 == 0:
            log(f"pairs: {i + 1}/{n_inst} instances, {time.time() - t0:.1f} s")
    return {"ops": ops, "r": R, "e": E, "inst": inst, "size": size}


def train(pairs, steps=1500, batch=8, lr=1e-3, seed=0, params=None, log=None, log_every=100):
    """Adam on sum_i ||N(r_i) - e_i/sigma_i||^2 / ||e_i/sigma_i||^2 over random
    batches of the pairs.  Returns (params, loss history)."""
    import torch
    size = pairs["size"]
    dev = pairs["r"].device
    net = UNet(batch, size, size, dev.index or 0)
    try:
        net.set_params(init_params(seed) if params is None else params)
        rng = np.random.Generator(np.random.PCG64(seed + 1))
        sig = torch.zeros(batch, dtype=torch.float32, device=dev)
        tgt = torch.zeros((batch, size, size), dtype=torch.float32, device=dev)
        msk = torch.zeros((batch, size, size), dtype=torch.uint8, device=dev)
        hist = []
        t0 = time.time()
        npairs = pairs["r"].shape[0]
        for step in range(1, steps + 1):
            idx = rng.integers(0, npairs, batch)
            for j, q in enumerate(idx):
                o = pairs["ops"][pairs["inst"][q]]
                net.features(j, size, size, pairs["r"][q], o[0], o[1], o[2], sig[j:j + 1])
                net.target(j, size, size, pairs["e"][q], o[2], sig[j:j + 1], tgt, msk)
            net.forward(torch.empty((batch, size, size), dtype=torch.float32, device=dev))
            L = net.loss(tgt, msk) / batch
            net.backward()
            net.adam(lr, step)
            hist.append(L)
            if log and (step % log_every == 0 or step == 1):
                log(f"step {step}: loss {np.mean(hist[-log_every:]):.4f} "
                    f"({time.time() - t0:.1f} s)")
        return net.get_params(), hist
    finally:
        net.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--instances", type=int, default=250)
    ap.add_argument("--iters", type=int, default=16)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--steps", type=int, default=1500)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=str(WEIGHTS))
    a = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)
    t0 = time.time()
    pairs = generate_pairs(a.instances, a.iters, a.size, log=log)
    t1 = time.time()
    params, hist = train(pairs, a.steps, a.batch, a.lr, a.seed, log=log)
    t2 = time.time()
    meta = {"instances": a.instances, "iters": a.iters, "size": a.size, "steps": a.steps,
            "batch": a.batch, "lr": a.lr, "seed": a.seed, "pairs_s": round(t1 - t0, 1),
            "train_s": round(t2 - t1, 1), "loss_first": float(np.mean(hist[:50])),
            "loss_last": float(np.mean(hist[-50:]))}
    save(params, a.out, meta)
    log(json.dumps(meta))


if __name__ == "__main__":
    main()
