"""Host side of the learned PPE initial guess / preconditioner scaling.

The network (include/mps_learned.h) is trained on the GPU by the library's own BF16
tensor-core forward/backward kernels and Adam kernel; this module only moves data and
loops over mini-batches.  Training data are (state features, converged pressure)
pairs that the plain FP64 Jacobi-CG solver itself produces (mps_solver_collect).
"""
import ctypes as C
import time

import numpy as np

from . import lib
from .types import MpsError

NPARAMS = 34946   # 12*128+128 + 2*(128*128+128) + 128*2+2
P = C.c_void_p
_SIGS = {
    "mps_gemm_bf16": (C.c_int, [C.c_int, C.c_int, C.c_int, P, C.c_int, C.c_int, P, C.c_int, C.c_int, P, C.c_int, P,
                                C.c_int, P, P, C.c_int, C.c_float, C.c_int, P]),
    "mps_gemm_bf16_variant": (C.c_int, [C.c_int, C.c_int, C.c_int, P, C.c_int, C.c_int, P, C.c_int, C.c_int, P,
                                        C.c_int, P, C.c_int, P, P, C.c_int, C.c_float, C.c_int, C.c_int, P]),
    "mps_mlp_create": (C.c_int, [C.c_int, C.c_ulonglong, C.POINTER(P)]),
    "mps_mlp_destroy": (None, [P]),
    "mps_mlp_set_params": (C.c_int, [P, P]),
    "mps_mlp_get_params": (C.c_int, [P, P]),
    "mps_mlp_forward": (C.c_int, [P, C.c_int, P, P, P]),
    "mps_mlp_forward_variant": (C.c_int, [P, C.c_int, P, P, C.c_int, P]),
    "mps_mlp_tc_timeouts": (C.c_int, [C.POINTER(C.c_uint)]),
    "mps_mlp_debug_wait_spins": (C.c_int, [C.c_longlong]),
    "mps_mlp_loss_grad": (C.c_int, [P, C.c_int, P, P, C.c_float, P, C.POINTER(C.c_float), P]),
    "mps_mlp_train_step": (C.c_int, [P, C.c_int, P, P, C.c_float, C.c_float, C.POINTER(C.c_float), P]),
}
_bound = False


def _lib():
    global _bound
    L = lib.load()
    if not _bound:
        for k, (r, a) in _SIGS.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _bound = True
    return L


def _check(rc, what):
    if rc != 0:
        raise MpsError(rc, f"{what} ({lib.load().mps_last_error().decode()})")


def gemm_bf16(M, N, K, A, lda, ta, B, ldb, tb, C_, ldc, Cb=None, ldcb=0, Cz=None, bias=None, act=0, beta=0.0,
              split=1, stream=None, variant=None):
    """Device pointers in, see mps_gemm_bf16 (variant 0 tcgen05, 1 mma.sync)."""
    if variant is None:
        _check(_lib().mps_gemm_bf16(M, N, K, A, lda, ta, B, ldb, tb, C_, ldc, Cb, ldcb, Cz, bias, act, beta, split,
                                    stream), "mps_gemm_bf16")
    else:
        _check(_lib().mps_gemm_bf16_variant(M, N, K, A, lda, ta, B, ldb, tb, C_, ldc, Cb, ldcb, Cz, bias, act, beta,
                                            split, variant, stream), "mps_gemm_bf16_variant")


class Mlp:
    def __init__(self, max_batch=8192, seed=1):
        h = P()
        _check(_lib().mps_mlp_create(max_batch, seed, C.byref(h)), "mps_mlp_create")
        self.h = h
        self.max_batch = max_batch

    def params(self) -> np.ndarray:
        p = np.zeros(NPARAMS, np.float32)
        _check(_lib().mps_mlp_get_params(self.h, p.ctypes.data), "mps_mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _check(_lib().mps_mlp_set_params(self.h, p.ctypes.data), "mps_mlp_set_params")

    def forward(self, X_dev, Y_dev, M, variant=None):
        """Y = MLP(X) on the device; variant None: the library's kernel (tcgen05), 0 the
        same, 1 the mma.sync cross-check kernel, 2..5 the tcgen05 kernel with 0..3 of
        every 4 pairs of hidden activations on the FMA pipe."""
        if variant is None:
            _check(_lib().mps_mlp_forward(self.h, M, X_dev, Y_dev, None), "mps_mlp_forward")
        else:
            _check(_lib().mps_mlp_forward_variant(self.h, M, X_dev, Y_dev, variant, None), "mps_mlp_forward_variant")

    @staticmethod
    def tc_timeouts() -> int:
        v = C.c_uint()
        _check(_lib().mps_mlp_tc_timeouts(C.byref(v)), "mps_mlp_tc_timeouts")
        return int(v.value)

    @staticmethod
    def debug_wait_spins(spins: int) -> None:
        """Polls of the tcgen05 inference kernel's MMA completion waits (negative: the
        default; 0: every wait runs out at once); clears the timeout flag."""
        _check(_lib().mps_mlp_debug_wait_spins(int(spins)), "mps_mlp_debug_wait_spins")

    def loss_grad(self, X_dev, T_dev, M, grad_dev, w1=0.25):
        loss = C.c_float()
        _check(_lib().mps_mlp_loss_grad(self.h, M, X_dev, T_dev, w1, grad_dev, C.byref(loss), None),
               "mps_mlp_loss_grad")
        return float(loss.value)

    def train_step(self, X_dev, T_dev, M, lr, w1=0.25, want_loss=False):
        loss = C.c_float()
        _check(_lib().mps_mlp_train_step(self.h, M, X_dev, T_dev, w1, lr, C.byref(loss) if want_loss else None, None),
               "mps_mlp_train_step")
        return float(loss.value) if want_loss else None

    def close(self):
        if getattr(self, "h", None):
            _lib().mps_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def collect_samples(scene, steps, precision="fp64", max_rows=400_000, seed=0, warm_start=2):
    """Runs the plain solver for `steps` steps and returns (features, targets) of its
    PPE solves: the network learns from (state, converged pressure) pairs of the
    plain solver itself.  The solver starts each solve from the warm start the learned
    solver will use (`warm_start`, the quadratic extrapolation of the FP32_IR default),
    so the features are taken there and the targets are the corrections to it."""
    from .solver import Solver
    s = Solver(scene, precision=precision, warm_start=warm_start)
    s.collect(True)
    fs, ts = [], []
    rng = np.random.default_rng(seed)
    for i in range(steps):
        s.step(i)
        f, t = s.learned_samples()
        if len(f) > max_rows // max(steps, 1):
            sel = rng.choice(len(f), size=max_rows // max(steps, 1), replace=False)
            f, t = f[sel], t[sel]
        fs.append(f)
        ts.append(t)
    s.close()
    return np.concatenate(fs), np.concatenate(ts)


def train(features, targets, epochs=4, batch=8192, lr=2e-3, seed=1, log=None, max_seconds=60.0):
    """Adam on the GPU (library kernels).  Returns (params, info)."""
    n = len(features)
    idx = np.random.default_rng(seed).permutation(n)
    n_val = max(1, n // 10)
    val, tr = idx[:n_val], idx[n_val:]
    X = lib.DeviceArray.from_host(np.ascontiguousarray(features, np.float32))
    T = lib.DeviceArray.from_host(np.ascontiguousarray(targets, np.float32))
    Xv = lib.DeviceArray.from_host(np.ascontiguousarray(features[val], np.float32))
    Tv = lib.DeviceArray.from_host(np.ascontiguousarray(targets[val], np.float32))
    mlp = Mlp(max_batch=max(batch, n_val), seed=seed)
    g = lib.DeviceArray((NPARAMS,), np.float32)
    loss0 = mlp.loss_grad(Xv.ptr, Tv.ptr, n_val, g.ptr)
    t0 = time.perf_counter()
    steps = 0
    rng = np.random.default_rng(seed + 1)
    Xb = lib.DeviceArray((batch, 12), np.float32)
    Tb = lib.DeviceArray((batch, 2), np.float32)
    for ep in range(epochs):
        perm = rng.permutation(tr)
        for b0 in range(0, len(perm) - batch + 1, batch):
            sel = perm[b0:b0 + batch]
            Xb.upload(features[sel])
            Tb.upload(targets[sel])
            mlp.train_step(Xb.ptr, Tb.ptr, batch, lr * (0.5 ** ep))
            steps += 1
        if time.perf_counter() - t0 > max_seconds:
            break
    loss1 = mlp.loss_grad(Xv.ptr, Tv.ptr, n_val, g.ptr)
    p = mlp.params()
    info = {"samples": int(n), "val_samples": int(n_val), "adam_steps": steps, "batch": batch,
            "val_loss_before": loss0, "val_loss_after": loss1, "train_seconds": time.perf_counter() - t0}
    if log is not None:
        log.append(f"learned: {info}")
    mlp.close()
    return p, info


def train_on_scene(scene, steps=6, log=None):
    """Data from `steps` plain FP64 steps of the scene (started as the learned solver
    starts, see collect_samples), then GPU training."""
    t0 = time.perf_counter()
    f, t = collect_samples(scene, steps)
    p, info = train(f, t, log=log)
    info["collect_seconds"] = time.perf_counter() - t0 - info["train_seconds"]
    return p, info
