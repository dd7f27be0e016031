"""Learned far-field correction: parameters, tensor-core training and inference.

A 6 -> 64 -> 64 -> 64 -> 2 GELU MLP (BF16 weights and activations, FP32
accumulation, tcgen05 kernels in libbh_gb300.so) maps the features of a
(target particle, far cell) pair to the dimensionless correction of the
monopole acceleration:

  features  u = dx / s, v = dy / s          (target -> cell centre of mass, cell edge s)
            qxx, qxy, qyy = I / (M s^2)     (second moments about the centre of mass)
            w = 1 / sqrt(u^2 + v^2)
  output    c such that  a_cell ~= a_monopole + G M / s * c

The box mass M enters as the exact linear scale of the correction.  Training
data are (target, cell) pairs produced by the method itself: the exact sum over
the cell's particles minus its monopole (see bh_learned_pairs).
"""
import ctypes

import numpy as np

from . import native

N_FEAT = 6


def _lib():
    L = native.load_library()
    if not getattr(L, "_mlp_typed", False):
        vp, ll, i, f = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_float
        L.bh_mlp_param_count.restype = i
        L.bh_mlp_image_bytes.restype = i
        L.bh_mlp_pack.argtypes = [vp, vp, vp]
        L.bh_mlp_pack.restype = i
        L.bh_mlp_forward.argtypes = [vp, i, ll, vp, vp, vp, vp, vp]
        L.bh_mlp_forward.restype = i
        L.bh_mlp_train_batch.argtypes = [vp, i, vp, ll, vp, vp, vp, vp, vp, vp]
        L.bh_mlp_train_batch.restype = i
        L.bh_mlp_adam.argtypes = [vp, vp, vp, vp, i, f, vp]
        L.bh_mlp_adam.restype = i
        L._mlp_typed = True
    return L


def init_params(seed=0):
    """Seeded initialisation (scaled uniform, zero biases) in the flat layout."""
    rng = np.random.default_rng(seed)
    p = np.zeros(10448, dtype=np.float32)

    def block(off, fan_in, shape, rows=None, cols=None):
        a = rng.uniform(-1, 1, size=shape) * np.sqrt(3.0 / fan_in)
        if rows is not None:
            a[rows:] = 0
        if cols is not None:
            a[:, cols:] = 0
        p[off:off + a.size] = a.reshape(-1)

    block(0, 6, (16, 64), rows=6)
    block(1088, 64, (64, 64))
    block(5248, 64, (64, 64))
    block(9408, 64, (64, 16), cols=2)
    return p


class LearnedCorrection:
    """Device-resident MLP parameters with tensor-core forward and training."""

    def __init__(self, params=None, device="cuda", seed=0):
        import torch

        self.torch = torch
        self.L = _lib()
        self.device = torch.device(device)
        assert self.L.bh_mlp_param_count() == 10448
        p = init_params(seed) if params is None else np.asarray(params, dtype=np.float32)
        self.params = torch.tensor(p, device=self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        self.image = torch.zeros(self.L.bh_mlp_image_bytes() + 256, dtype=torch.uint8, device=self.device)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        self.step_count = 0
        self.target_scale = 1.0
        self.pack()

    def _st(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream)

    def _img(self):
        off = (-self.image.data_ptr()) % 256
        return ctypes.c_void_p(self.image.data_ptr() + off)

    def _check(self, rc, what):
        if rc != 0:
            raise native.BHError(rc, what)

    def pack(self):
        self._check(self.L.bh_mlp_pack(ctypes.c_void_p(self.params.data_ptr()), self._img(),
                                       self._st()), "bh_mlp_pack")

    def check_errors(self):
        e = int(self.err.item())
        if e:
            self.err.zero_()
            raise native.BHError(native.BH_ERR_DEVICE, f"mlp device error flags 0x{e:x}")

    def forward(self, feats):
        """feats: (P, >=6) float32 device tensor -> (P, 2) float32."""
        torch = self.torch
        f = feats.to(self.device, torch.float32).contiguous()
        out = torch.empty((f.shape[0], 2), dtype=torch.float32, device=self.device)
        self._check(self.L.bh_mlp_forward(ctypes.c_void_p(f.data_ptr()), f.shape[1], f.shape[0],
                                          self._img(), ctypes.c_void_p(self.params.data_ptr()),
                                          ctypes.c_void_p(out.data_ptr()),
                                          ctypes.c_void_p(self.err.data_ptr()), self._st()),
                    "bh_mlp_forward")
        return out

    def grad_batch(self, feats, targets):
        """Accumulate the gradient of mean((y - t)^2) over the batch; returns the loss."""
        torch = self.torch
        f = feats.to(self.device, torch.float32).contiguous()
        t = targets.to(self.device, torch.float32).contiguous()
        self.loss.zero_()
        self._check(self.L.bh_mlp_train_batch(
            ctypes.c_void_p(f.data_ptr()), f.shape[1], ctypes.c_void_p(t.data_ptr()), f.shape[0],
            self._img(), ctypes.c_void_p(self.params.data_ptr()),
            ctypes.c_void_p(self.grad.data_ptr()), ctypes.c_void_p(self.loss.data_ptr()),
            ctypes.c_void_p(self.err.data_ptr()), self._st()), "bh_mlp_train_batch")
        return self.loss

    def adam_step(self, lr):
        self.step_count += 1
        self._check(self.L.bh_mlp_adam(ctypes.c_void_p(self.params.data_ptr()),
                                       ctypes.c_void_p(self.m.data_ptr()),
                                       ctypes.c_void_p(self.v.data_ptr()),
                                       ctypes.c_void_p(self.grad.data_ptr()), self.step_count,
                                       float(lr), self._st()), "bh_mlp_adam")
        self.pack()

    def train(self, feats, targets, epochs=4, batch=65536, lr=2e-3, seed=0, log=None):
        """Mini-batch Adam on device tensors; returns the per-epoch mean loss."""
        torch = self.torch
        n = feats.shape[0]
        gen = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        for ep in range(epochs):
            perm = torch.randperm(n, generator=gen).to(self.device)
            tot = 0.0
            nb = 0
            lr_ep = lr * (0.5 ** ep)
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                loss = self.grad_batch(feats[idx], targets[idx])
                self.adam_step(lr_ep)
                tot += float(loss.item()) / (batch * 2)
                nb += 1
            hist.append(tot / max(nb, 1))
            if log:
                log(f"epoch {ep}: loss {hist[-1]:.4e}")
        self.check_errors()
        return hist

    def state(self):
        return {"params": self.params.cpu().numpy(), "target_scale": self.target_scale}


def generate_pairs(systems, grid, theta_hi, theta_lo, n_pairs, max_level=5, targets_per_item=8,
                   softening=1e-4, device="cuda", seed=0):
    """Training rows made by the method: for each (x, y, m, vx, vy) system, build the tree and
    collect (target, band cell) rows until n_pairs rows exist.  Returns device tensors
    feats (n, 8) and targets (n, 2)."""
    import torch

    feats = torch.zeros((n_pairs, 8), dtype=torch.float32, device=device)
    targs = torch.zeros((n_pairs, 2), dtype=torch.float32, device=device)
    counter = torch.zeros(1, dtype=torch.int32, device=device)
    per_sys = max(1, n_pairs // max(1, len(systems)))
    for k, s in enumerate(systems):
        prm = native.make_params(1.0, 1e-5, softening, 0.0, theta_hi, 0, native.BH_PREC_FP32_KAHAN)
        plan = native.Plan([len(s[0])], [grid], prm, device=device)
        plan.load(*s)
        plan.create_tree()
        plan.summarize()
        goal = min(n_pairs, (k + 1) * per_sys if k + 1 < len(systems) else n_pairs)
        offset, stride = (seed + k) % 7, 7
        rounds = 0
        while int(counter.item()) < goal and rounds < 7:
            plan.learned_pairs(theta_hi, theta_lo, goal, max_level=max_level,
                               item_offset=(offset + rounds) % stride, item_stride=stride,
                               targets_per_item=targets_per_item, feats=feats, targets=targs,
                               counter=counter)
            rounds += 1
        # rows past the capacity were counted but not written: the next system appends
        # right after the last written row
        counter.clamp_(max=goal)
        plan.error_flags()
        plan.close()
    n = min(int(counter.item()), n_pairs)
    return feats[:n], targs[:n]


def fold_output_scale(mlp, scale):
    """Multiply the network output by `scale` (last layer weights and bias)."""
    p = mlp.params
    p[9408:10432] *= scale
    p[10432:10448] *= scale
    mlp.pack()


def fold_input_standardisation(mlp, mu, sigma):
    """The network was trained on (x - mu) / sigma; fold that into W1 and b1 so the
    kernels take raw features: W1' = W1 / sigma, b1' = b1 - (mu / sigma) W1."""
    import torch

    p = mlp.params
    W1 = p[0:1024].view(16, 64)
    mu_t = torch.zeros(16, device=p.device)
    sg_t = torch.ones(16, device=p.device)
    mu_t[:N_FEAT] = torch.as_tensor(mu, dtype=torch.float32, device=p.device)
    sg_t[:N_FEAT] = torch.as_tensor(sigma, dtype=torch.float32, device=p.device)
    b1 = p[1024:1088]
    b1 -= (mu_t / sg_t) @ W1
    W1 /= sg_t[:, None]
    mlp.pack()


def quadrupole_prediction(feats):
    """Analytic 2D quadrupole term of the (target, cell) correction in the same units:
    (exact - monopole) * s / M ~= Re, Im of (qxx - qyy - 2i qxy) / (u - i v)^3."""
    import torch

    u, v = feats[:, 0].double(), feats[:, 1].double()
    a, b = (feats[:, 2] - feats[:, 4]).double(), (-2.0 * feats[:, 3]).double()
    z = torch.complex(u, -v)
    c = torch.complex(a, b) / z ** 3
    return torch.stack([c.real, c.imag], dim=1).float()


def train_correction(systems, grid, theta_hi=0.8, theta_lo=0.5, n_pairs=1 << 20, epochs=4,
                     batch=4096, lr=3e-3, seed=0, device="cuda", log=None):
    """Generate pairs, train the MLP on standardised features and normalised targets, fold
    both normalisations into the weights."""
    import torch

    feats, targs = generate_pairs(systems, grid, theta_hi, theta_lo, n_pairs, seed=seed,
                                  device=device)
    mu = feats[:, :N_FEAT].mean(0)
    sigma = feats[:, :N_FEAT].std(0) + 1e-12
    fstd = feats.clone()
    fstd[:, :N_FEAT] = (feats[:, :N_FEAT] - mu) / sigma
    scale = float(targs.std()) + 1e-30
    mlp = LearnedCorrection(device=device, seed=seed)
    hist = mlp.train(fstd, targs / scale, epochs=epochs, batch=min(batch, feats.shape[0]),
                     lr=lr, seed=seed, log=log)
    fold_input_standardisation(mlp, mu.cpu().numpy(), sigma.cpu().numpy())
    fold_output_scale(mlp, scale)
    mlp.target_scale = scale
    with torch.no_grad():
        den = float((targs ** 2).mean())
        pred = mlp.forward(feats)
        resid = float(((pred - targs) ** 2).mean()) / den
        quad = float(((quadrupole_prediction(feats) - targs) ** 2).mean()) / den
    return mlp, {"pairs": int(feats.shape[0]), "loss_history": hist, "scale": scale,
                 "relative_mse": resid, "quadrupole_relative_mse": quad}
