"""ctypes binding of libbh_gb300.so (the C ABI in include/bh_gb300.h).

There is no fallback: if the library is missing or cannot be loaded, every
entry point raises ``NativeLibraryError``.  Device memory comes from PyTorch
(one uint8 workspace tensor per plan); streams are torch CUDA streams.
"""
import ctypes
import os

import numpy as np

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libbh_gb300.so")

BH_OK = 0
BH_ERR_INVALID = 1
BH_ERR_CUDA = 2
BH_ERR_WORKSPACE = 3
BH_ERR_DEVICE = 4
BH_ERR_TIMEOUT = 5

BH_DEV_NAN_POSITION = 1
BH_DEV_LIST_OVERFLOW = 2
BH_DEV_BAD_KEY = 4
BH_DEV_WAIT_TIMEOUT = 8

BH_PREC_FP32 = 0
BH_PREC_FP32_KAHAN = 1
BH_PREC_FP64 = 2

BH_FLAG_LEARNED = 1
BH_FLAG_WALK = 2
BH_STREAM_DENSE_MIN = 64  # include/bh_gb300.h
BH_STREAM_QUAD_MIN = 128

# every symbol include/bh_gb300.h declares
EXPORTS = (
    "bh_grid_dim", "bh_plan_create", "bh_plan_destroy", "bh_last_error", "bh_workspace_size",
    "bh_bind", "bh_load", "bh_load_records", "bh_store_records", "bh_store", "bh_create_tree",
    "bh_summarize", "bh_evaluate", "bh_timestep", "bh_step", "bh_step_graph", "bh_error_flags",
    "bh_pair_counts", "bh_box_moments", "bh_grid_info", "bh_direct_sample", "bh_diagnostics",
    "bh_kernels_per_step", "bh_mlp_param_count", "bh_mlp_image_bytes", "bh_mlp_pack",
    "bh_mlp_forward", "bh_mlp_train_batch", "bh_mlp_adam", "bh_set_correction", "bh_learned_pairs",
    "bh_direct_sum_noalloc", "bh_generate", "bh_graph_kernel_nodes", "bh_set_kernel_timing",
    "bh_force_kernel_ms", "bh_corrected_pairs", "bh_set_grid", "bh_leaf_moments", "bh_set_leaf_moments",
)
BH_GEN_UNIFORM, BH_GEN_GAUSS, BH_GEN_CLUSTER = 0, 1, 2
BH_NOALLOC_MAX_TARGETS = 4096


class NativeLibraryError(RuntimeError):
    pass


class BHError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [
        ("grav_constant", ctypes.c_double),
        ("tick_seconds", ctypes.c_double),
        ("softening", ctypes.c_double),
        ("cutoff_r2", ctypes.c_double),
        ("theta", ctypes.c_double),
        ("group_dim", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("flags", ctypes.c_int),
        ("tune", ctypes.c_int),
        ("correction_theta", ctypes.c_double),
        ("dense_min", ctypes.c_int),
        ("quad_min", ctypes.c_int),
    ]


_lib = None


def load_library(path=None):
    """Load and type the native library (once)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise NativeLibraryError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            " (there is no CPU fallback)")
    try:
        L = ctypes.CDLL(path)
    except OSError as e:
        raise NativeLibraryError(f"cannot load {path}: {e}") from e
    vp, ll, i, d = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_double
    pll = ctypes.POINTER(ll)
    pi = ctypes.POINTER(i)
    L.bh_grid_dim.argtypes = [ll, i]
    L.bh_grid_dim.restype = i
    L.bh_plan_create.argtypes = [ctypes.POINTER(vp), i, pll, pi, ctypes.POINTER(Params)]
    L.bh_plan_destroy.argtypes = [vp]
    L.bh_last_error.argtypes = [vp]
    L.bh_last_error.restype = ctypes.c_char_p
    L.bh_workspace_size.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
    L.bh_bind.argtypes = [vp, vp, ctypes.c_size_t, vp]
    L.bh_load.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.bh_load_records.argtypes = [vp, vp, vp]
    L.bh_store_records.argtypes = [vp, vp, vp]
    L.bh_store.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    for name in ("bh_create_tree", "bh_summarize", "bh_evaluate", "bh_timestep"):
        getattr(L, name).argtypes = [vp, vp]
    L.bh_step.argtypes = [vp, i, vp]
    L.bh_step_graph.argtypes = [vp, i, vp]
    L.bh_error_flags.argtypes = [vp, ctypes.POINTER(ctypes.c_uint), vp]
    L.bh_pair_counts.argtypes = [vp, pll, pll, vp]
    L.bh_box_moments.argtypes = [vp, i, vp, vp]
    L.bh_grid_info.argtypes = [vp, i, ctypes.POINTER(d), vp]
    L.bh_direct_sample.argtypes = [vp, i, vp, ll, vp, vp, vp]
    L.bh_diagnostics.argtypes = [vp, i, i, vp, vp]
    L.bh_kernels_per_step.argtypes = [vp, pi]
    L.bh_graph_kernel_nodes.argtypes = [vp, pi]
    L.bh_set_kernel_timing.argtypes = [vp, i]
    L.bh_corrected_pairs.argtypes = [vp, pll, vp]
    L.bh_set_grid.argtypes = [vp, i, ctypes.POINTER(d), vp]
    L.bh_leaf_moments.argtypes = [vp, i, vp, vp]
    L.bh_set_leaf_moments.argtypes = [vp, i, vp, vp]
    L.bh_force_kernel_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
    L.bh_set_correction.argtypes = [vp, vp, vp]
    L.bh_direct_sum_noalloc.argtypes = [vp, vp, vp, ll, vp, ll, d, d, vp, vp, vp]
    L.bh_learned_pairs.argtypes = [vp, d, d, i, ll, ll, i, vp, vp, vp, ll, vp]
    L.bh_generate.argtypes = [i, ll, ctypes.c_ulonglong, vp, vp, vp, vp, vp, vp]
    for name in EXPORTS:
        f = getattr(L, name)
        if name not in ("bh_last_error",):
            f.restype = i
    _lib = L
    return L


def grid_dim(n, max_particles_per_box):
    return load_library().bh_grid_dim(int(n), int(max_particles_per_box))


def generate(distribution, n, seed, device="cuda"):
    """n particles drawn on the device (bh_generate): dict of FP64 tensors x, y, m, vx, vy."""
    import torch

    L = load_library()
    out = {k: torch.empty(int(n), dtype=torch.float64, device=device) for k in ("x", "y", "m", "vx", "vy")}
    st = torch.cuda.current_stream(out["x"].device).cuda_stream
    rc = L.bh_generate(int(distribution), int(n), int(seed) & 0xFFFFFFFFFFFFFFFF,
                       *[_ptr(out[k]) for k in ("x", "y", "m", "vx", "vy")], ctypes.c_void_p(st))
    if rc != BH_OK:
        raise BHError(rc, (L.bh_last_error(None) or b"").decode())
    return out


def make_params(grav_constant=1.0, tick_seconds=0.005, softening=0.0, cutoff_r2=1e-5,
                theta=0.0, group_dim=0, precision=BH_PREC_FP32_KAHAN, flags=0, tune=0,
                correction_theta=0.0, dense_min=0, quad_min=0):
    return Params(float(grav_constant), float(tick_seconds), float(softening), float(cutoff_r2),
                  float(theta), int(group_dim), int(precision), int(flags), int(tune),
                  float(correction_theta), int(dense_min), int(quad_min))


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class Plan:
    """One plan = nsys independent systems stepped together on one GPU.

    ``n`` and ``grid_dims`` are sequences (one entry per system).  Device
    memory: one torch.uint8 workspace tensor on ``device``.
    """

    def __init__(self, n, grid_dims, params, device=None, stream=None):
        import torch

        self._torch = torch
        L = load_library()
        self.L = L
        n = [int(v) for v in n]
        g = [int(v) for v in grid_dims]
        if len(n) != len(g) or not n:
            raise ValueError("n and grid_dims must be non-empty and of equal length")
        self.nsys = len(n)
        self.n = n
        self.n_total = sum(n)
        self.params = params
        self.device = torch.device(device if device is not None else "cuda")
        h = ctypes.c_void_p()
        na = (ctypes.c_longlong * len(n))(*n)
        ga = (ctypes.c_int * len(g))(*g)
        rc = L.bh_plan_create(ctypes.byref(h), len(n), na, ga, ctypes.byref(params))
        if rc != BH_OK:
            raise BHError(rc, L.bh_last_error(None).decode())
        self.h = h
        sz = ctypes.c_size_t()
        self._check(L.bh_workspace_size(h, ctypes.byref(sz)))
        self.workspace_bytes = sz.value
        with torch.cuda.device(self.device):
            self.workspace = torch.empty(self.workspace_bytes + 256, dtype=torch.uint8,
                                         device=self.device)
        off = (-self.workspace.data_ptr()) % 256
        self._ws_ptr = self.workspace.data_ptr() + off
        self.stream = stream
        with torch.cuda.device(self.device):
            self._check(L.bh_bind(h, ctypes.c_void_p(self._ws_ptr), self.workspace_bytes,
                                  self._st()))

    # ------------------------------------------------------------ plumbing
    def _st(self):
        torch = self._torch
        s = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        return ctypes.c_void_p(s.cuda_stream)

    def _check(self, rc):
        if rc != BH_OK:
            raise BHError(rc, self.L.bh_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.bh_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _dev(self, a):
        torch = self._torch
        t = torch.as_tensor(a, dtype=torch.float64)
        return t.to(self.device).contiguous()

    # ------------------------------------------------------------ state
    def load(self, x, y, m, vx, vy):
        """Upload concatenated particle arrays (pid order)."""
        ts = [self._dev(a) for a in (x, y, m, vx, vy)]
        for t in ts:
            if t.numel() != self.n_total:
                raise ValueError(f"expected {self.n_total} values, got {t.numel()}")
        self._check(self.L.bh_load(self.h, *[_ptr(t) for t in ts], self._st()))
        self._keep = ts  # alive until the async upload ran

    def load_records(self, records):
        """Upload an N x 10 float64 reference record array (numpy or tensor)."""
        t = self._dev(records)
        if t.dim() != 2 or t.shape[1] != 10 or t.shape[0] != self.n_total:
            raise ValueError("records must be N x 10 float64")
        self._check(self.L.bh_load_records(self.h, _ptr(t), self._st()))
        self._keep = [t]

    def store_records(self):
        """N x 10 float64 device tensor in pid order."""
        torch = self._torch
        out = torch.empty((self.n_total, 10), dtype=torch.float64, device=self.device)
        self._check(self.L.bh_store_records(self.h, _ptr(out), self._st()))
        return out

    def store(self):
        """dict of device tensors x, y, vx, vy, ax, ay in pid order."""
        torch = self._torch
        out = {k: torch.empty(self.n_total, dtype=torch.float64, device=self.device)
               for k in ("x", "y", "vx", "vy", "ax", "ay")}
        self._check(self.L.bh_store(self.h, *[_ptr(out[k]) for k in
                                              ("x", "y", "vx", "vy", "ax", "ay")], self._st()))
        return out

    # ------------------------------------------------------------ phases
    def create_tree(self):
        self._check(self.L.bh_create_tree(self.h, self._st()))

    def summarize(self):
        self._check(self.L.bh_summarize(self.h, self._st()))

    def evaluate(self):
        self._check(self.L.bh_evaluate(self.h, self._st()))

    def timestep(self):
        self._check(self.L.bh_timestep(self.h, self._st()))

    def step(self, nsteps=1):
        self._check(self.L.bh_step(self.h, int(nsteps), self._st()))

    def step_graph(self, nsteps=1):
        self._check(self.L.bh_step_graph(self.h, int(nsteps), self._st()))

    # ------------------------------------------------------------ checks
    def error_flags(self, raise_on_error=True):
        f = ctypes.c_uint(0)
        rc = self.L.bh_error_flags(self.h, ctypes.byref(f), self._st())
        if rc not in (BH_OK, BH_ERR_DEVICE):
            self._check(rc)
        if raise_on_error and f.value:
            raise BHError(BH_ERR_DEVICE, f"device error flags 0x{f.value:x}")
        return f.value

    def set_correction(self, mlp):
        """Bind a LearnedCorrection (barneshut.gb300.learned) used when the plan's
        params carry BH_FLAG_LEARNED."""
        self._mlp = mlp
        self._check(self.L.bh_set_correction(self.h, mlp._img(),
                                             ctypes.c_void_p(mlp.params.data_ptr())))

    def learned_pairs(self, theta_hi, theta_lo, capacity, max_level=5, item_offset=0,
                      item_stride=16, targets_per_item=8, feats=None, targets=None, counter=None):
        """Training rows from the current tree (after create_tree + summarize).
        Returns (feats (cap, 8), targets (cap, 2), counter tensor)."""
        torch = self._torch
        if feats is None:
            feats = torch.zeros((capacity, 8), dtype=torch.float32, device=self.device)
            targets = torch.zeros((capacity, 2), dtype=torch.float32, device=self.device)
            counter = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._check(self.L.bh_learned_pairs(
            self.h, float(theta_hi), float(theta_lo), int(max_level), int(item_offset),
            int(item_stride), int(targets_per_item), _ptr(feats), _ptr(targets), _ptr(counter),
            int(capacity), self._st()))
        return feats, targets, counter

    def kernels_per_step(self):
        c = ctypes.c_int()
        self._check(self.L.bh_kernels_per_step(self.h, ctypes.byref(c)))
        return c.value

    def graph_kernel_nodes(self):
        """Kernel nodes of the step graph captured by the last step_graph call."""
        c = ctypes.c_int()
        self._check(self.L.bh_graph_kernel_nodes(self.h, ctypes.byref(c)))
        return c.value

    def set_grid(self, extents, sys=0):
        """Fix the grid of system `sys` to the whole system's extents (min x, min y, max x,
        max y); None returns to the plan's own bounding box."""
        if extents is None:
            self._check(self.L.bh_set_grid(self.h, sys, None, self._st()))
        else:
            e = (ctypes.c_double * 4)(*[float(v) for v in extents])
            self._check(self.L.bh_set_grid(self.h, sys, e, self._st()))

    def leaf_moments(self, sys=0):
        """(G, G, 6) device tensor: the last summarize's leaf moments (M, Sx, Sy, Sxx, Sxy, Syy
        about each box origin; the second moments only with the learned correction, zeros
        otherwise)."""
        torch = self._torch
        G = self.grid_info(sys)["grid_dim"]
        out = torch.empty((G, G, 6), dtype=torch.float64, device=self.device)
        self._check(self.L.bh_leaf_moments(self.h, sys, _ptr(out), self._st()))
        return out

    def set_leaf_moments(self, leaf, sys=0):
        """Replace the leaf moments of system `sys` (device (G, G, 6) FP64) and rebuild the
        pyramid above them."""
        leaf = self._torch.as_tensor(leaf, dtype=self._torch.float64, device=self.device).contiguous()
        self._check(self.L.bh_set_leaf_moments(self.h, sys, _ptr(leaf), self._st()))
        self._keep = leaf  # alive until the copy has run

    def set_kernel_timing(self, enable=True):
        """Record CUDA events around the force kernel of every later eager evaluate()."""
        self._check(self.L.bh_set_kernel_timing(self.h, 1 if enable else 0))

    def force_kernel_ms(self):
        """Duration of the force kernel of the last timed evaluate() (waits for it)."""
        v = ctypes.c_float()
        self._check(self.L.bh_force_kernel_ms(self.h, ctypes.byref(v)))
        return v.value

    def pair_counts(self):
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        self._check(self.L.bh_pair_counts(self.h, ctypes.byref(a), ctypes.byref(b), self._st()))
        return a.value, b.value

    def corrected_pairs(self):
        """(target, cell) pairs the learned correction evaluated in the last step."""
        a = ctypes.c_longlong()
        self._check(self.L.bh_corrected_pairs(self.h, ctypes.byref(a), self._st()))
        return a.value

    def box_moments(self, sys=0):
        """(G, G, 3) device tensor of leaf (cx, cy, M) from the last summarize."""
        torch = self._torch
        G = self.grid_info(sys)["grid_dim"]
        out = torch.empty((G, G, 3), dtype=torch.float64, device=self.device)
        self._check(self.L.bh_box_moments(self.h, int(sys), _ptr(out), self._st()))
        return out

    def grid_info(self, sys=0):
        o = (ctypes.c_double * 5)()
        self._check(self.L.bh_grid_info(self.h, int(sys), o, self._st()))
        return {"min_x": o[0], "min_y": o[1], "step": o[2], "grid_dim": int(o[3]), "n": int(o[4])}

    def direct_sample(self, targets, sys=0):
        """FP64 direct-sum accelerations on the device for pid targets."""
        torch = self._torch
        t = torch.as_tensor(np.asarray(targets, dtype=np.int64)).to(self.device)
        ax = torch.empty(t.numel(), dtype=torch.float64, device=self.device)
        ay = torch.empty_like(ax)
        self._check(self.L.bh_direct_sample(self.h, int(sys), _ptr(t), t.numel(), _ptr(ax),
                                            _ptr(ay), self._st()))
        return ax, ay

    def diagnostics(self, sys=0, potential=False):
        """(kinetic, momentum_x, momentum_y, potential) as floats (syncs)."""
        torch = self._torch
        out = torch.zeros(4, dtype=torch.float64, device=self.device)
        self._check(self.L.bh_diagnostics(self.h, int(sys), 1 if potential else 0, _ptr(out),
                                          self._st()))
        return tuple(float(v) for v in out.cpu())
