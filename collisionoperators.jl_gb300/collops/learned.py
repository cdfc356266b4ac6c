"""Learned warm start of the implicit step.

A small MLP (15 -> 64 -> 64 -> 64 -> 2, GELU, BF16 weights, FP32 accumulation;
the kernels are this library's own, see co_mlp.cu) maps per-marker features at
the start of a step to the correction of the explicit predictor,
    delta = (v_converged - v_Euler) / dt^2,
the form of warm start the reference planned ("Euler + dt^2 * delta" MLP
correction, Parameters.jl:108-112; its warmstart_nn.jl is not in the tree).
The feature and output normalisation are held by the network itself and
applied inside its forward kernel.

The fixed-point map decides: the step starts from whichever of the learned
proposal, the explicit predictor and the previous-step state has the smallest
first Picard residual, and the unmodified solver judges convergence
(co_step_learned, one C-ABI call for the whole step).

Training data comes from the solver itself: `generate_pairs` runs time steps
and records (features at the step start, delta of the step) for the steps whose
solve converged.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import CollopsError, CoOpts, Workspace, _check, _p, load_library

N_IN, N_OUT = 15, 2   # features per marker (co_warmstart_features_dev), outputs


class MLP:
    """The network on one device (co_mlp_*)."""

    def __init__(self, seed: int = 0, device: int = 0, n_in: int = N_IN, n_out: int = N_OUT):
        self.lib = load_library()
        h = C.c_void_p()
        self.h = None
        _check(self.lib.co_mlp_create(n_in, n_out, seed, device, C.byref(h)), "co_mlp_create")
        self.h = h
        P = C.c_int()
        _check(self.lib.co_mlp_num_params(self.h, C.byref(P)), "co_mlp_num_params")
        self.P = P.value
        self.n_in, self.n_out = n_in, n_out

    def close(self):
        if self.h is not None:
            self.lib.co_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.P, dtype=np.float32)
        _check(self.lib.co_mlp_get_params(self.h, out.ctypes.data_as(C.POINTER(C.c_float))),
               "co_mlp_get_params")
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.P
        _check(self.lib.co_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))),
               "co_mlp_set_params")

    def _rows(self, X, cols: int, name: str) -> int:
        """The kernels take row pointers and a row count only: check the layout
        (contiguous float32 CUDA rows of exactly `cols`) before every call."""
        import torch
        if not (isinstance(X, torch.Tensor) and X.is_cuda and X.dtype == torch.float32 and
                X.dim() == 2 and X.shape[1] == cols and X.is_contiguous()):
            raise CollopsError(f"{name}: expected a contiguous float32 CUDA tensor (B, {cols}), "
                               f"got {getattr(X, 'shape', None)} "
                               f"{getattr(X, 'dtype', type(X).__name__)}")
        return X.shape[0]

    def forward(self, X, Y, stream: int = 0) -> None:
        """X (B, n_in) and Y (B, n_out): float32 CUDA tensors; enqueued on `stream`
        (a cudaStream_t as an int, 0 = the legacy default stream)."""
        B = self._rows(X, self.n_in, "X")
        if self._rows(Y, self.n_out, "Y") != B:
            raise CollopsError("forward: X and Y row counts differ")
        _check(self.lib.co_mlp_forward(self.h, X.data_ptr(), B, Y.data_ptr(),
                                       C.c_void_p(stream or None)), "co_mlp_forward")

    def gradients(self, X, T):
        B = self._rows(X, self.n_in, "X")
        if self._rows(T, self.n_out, "T") != B:
            raise CollopsError("gradients: X and T row counts differ")
        g = np.zeros(self.P, dtype=np.float32)
        loss = C.c_float()
        _check(self.lib.co_mlp_gradients(self.h, X.data_ptr(), T.data_ptr(), X.shape[0],
                                         g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)),
               "co_mlp_gradients")
        return g, loss.value

    def train_step(self, X, T, lr: float) -> float:
        B = self._rows(X, self.n_in, "X")
        if self._rows(T, self.n_out, "T") != B:
            raise CollopsError("train_step: X and T row counts differ")
        loss = C.c_float()
        _check(self.lib.co_mlp_train_step(self.h, X.data_ptr(), T.data_ptr(), X.shape[0], lr,
                                          C.byref(loss)), "co_mlp_train_step")
        return loss.value


def features(ws: Workspace, opts: CoOpts, v, w, S0: float, dt: float):
    """(X float32 (N, 15), v_pred, ||G(v_pred) - v_pred||) on the device for
    markers v (torch (2, N)) whose projection has entropy S0."""
    import torch
    N = v.shape[1]
    X = torch.empty((N, N_IN), dtype=torch.float32, device=v.device)
    vp = torch.empty_like(v)
    rp = C.c_double()
    _check(ws.lib.co_warmstart_features_dev(ws.h, C.byref(opts), v.data_ptr(), w.data_ptr(), N,
                                            S0, dt, vp.data_ptr(), X.data_ptr(), C.byref(rp)),
           "co_warmstart_features_dev")
    return X, vp, rp.value


class WarmStart:
    """Normalisation + network; `propose` implements the learned warm start."""

    def __init__(self, mlp: MLP | None = None, device: int = 0, relax: float = 1.0):
        self.mlp = mlp or MLP(device=device)
        self.xm = np.zeros(self.mlp.n_in)
        self.xs = np.ones(self.mlp.n_in)
        self.tm = np.zeros(self.mlp.n_out)
        self.ts = np.ones(self.mlp.n_out)
        # under-relaxation of the proposal: v = v_pred + relax dt^2 delta
        self.relax = float(relax)

    def _push_normalization(self) -> None:
        """Hand the normalisation to the network: its forward kernel then takes
        raw features and returns relax * delta itself (co_mlp_set_normalization;
        the output mean and scale carry the relaxation factor)."""
        d = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
        xm, xs = d(self.xm), d(self.xs)
        tm, ts = d(self.tm * self.relax), d(self.ts * self.relax)
        _check(self.mlp.lib.co_mlp_set_normalization(self.mlp.h, _p(xm), _p(xs), _p(tm), _p(ts)),
               "co_mlp_set_normalization")

    def validation_loss(self, X: np.ndarray, T: np.ndarray, device: int = 0) -> float:
        """Mean squared error of the normalised prediction on (X, T) (co_mlp_gradients
        computes the loss; the gradient is discarded)."""
        import torch
        Xn = torch.from_numpy(((X - self.xm) / self.xs).astype(np.float32)).cuda(device)
        Tn = torch.from_numpy(((T - self.tm) / self.ts).astype(np.float32)).cuda(device)
        _g, loss = self.mlp.gradients(Xn.contiguous(), Tn.contiguous())
        return float(loss)

    def fit(self, X: np.ndarray, T: np.ndarray, epochs: int = 20, batch: int = 8192,
            lr: float = 2e-3, seed: int = 0, device: int = 0):
        """Train on the GPU with the library's kernels; returns the loss history."""
        import torch
        self.xm, self.xs = X.mean(0), X.std(0) + 1e-12
        self.tm, self.ts = T.mean(0), T.std(0) + 1e-30
        Xn = torch.from_numpy(((X - self.xm) / self.xs).astype(np.float32)).cuda(device)
        Tn = torch.from_numpy(((T - self.tm) / self.ts).astype(np.float32)).cuda(device)
        rng = np.random.default_rng(seed)
        hist = []
        n = X.shape[0]
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(n)).cuda(device)
            tot, cnt = 0.0, 0
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                tot += self.mlp.train_step(Xn[idx].contiguous(), Tn[idx].contiguous(),
                                           lr * (0.5 ** (ep // max(1, epochs // 3))))
                cnt += 1
            hist.append(tot / max(cnt, 1))
        self._push_normalization()
        return hist

    def predict_delta(self, X, stream: int = 0):
        """Raw features (float32 CUDA tensor (B, 15)) -> delta (B, 2), both the
        normalisation and the network in the library's forward kernel, on
        `stream` (a cudaStream_t as an int)."""
        import torch
        Y = torch.empty((X.shape[0], N_OUT), dtype=torch.float32, device=X.device)
        self.mlp.forward(X.contiguous(), Y, stream)
        return Y

    def propose(self, ws: Workspace, opts: CoOpts, v, w, S0: float, dt: float, v1_out,
                alt_out=None):
        """Fill v1_out with the initial iterate: the learned proposal if its first
        residual is smaller than the predictor's, else the predictor (and alt_out,
        if given, with the other one). Returns (used_learned, residual_learned,
        residual_predictor)."""
        import torch
        X, vp, rp_pred = features(ws, opts, v, w, S0, dt)
        # features() returns after the context stream has drained; the network and
        # everything after it stay on that stream, so co_warmstart_apply_dev sees Y
        Y = self.predict_delta(X, ws.stream())
        N = v.shape[1]
        vl = torch.empty_like(v)
        sc = np.ones(N_OUT)       # the network returns delta itself
        sh = np.zeros(N_OUT)
        _check(ws.lib.co_warmstart_apply_dev(ws.h, vp.data_ptr(), Y.data_ptr(), N, dt, _p(sc),
                                             _p(sh), vl.data_ptr()), "co_warmstart_apply_dev")
        rl = C.c_double()
        _check(ws.lib.co_picard_residual_dev(ws.h, C.byref(opts), vl.data_ptr(), v.data_ptr(),
                                             w.data_ptr(), N, S0, dt, C.byref(rl)),
               "co_picard_residual_dev")
        use = rl.value < rp_pred
        with torch.cuda.stream(torch.cuda.ExternalStream(ws.stream(), device=v.device)):
            v1_out.copy_(vl if use else vp)
            if alt_out is not None:
                alt_out.copy_(vp if use else vl)
        return use, rl.value, rp_pred

    def save(self, path: str) -> None:
        np.savez_compressed(path, params=self.mlp.get_params(), xm=self.xm, xs=self.xs,
                            tm=self.tm, ts=self.ts)

    @classmethod
    def load(cls, path: str, device: int = 0, relax: float = 1.0) -> "WarmStart":
        """The trained network and its normalisation from `path`; relax < 1
        under-relaxes the proposal (v_pred + relax dt^2 delta)."""
        z = np.load(path)
        ws = cls(device=device, relax=relax)
        if z["params"].size != ws.mlp.P or z["xm"].size != ws.mlp.n_in:
            raise CollopsError(f"{path}: {z['xm'].size}-feature network, this library builds "
                               f"{ws.mlp.n_in} features per marker; retrain with "
                               "collops.train_warmstart")
        ws.mlp.set_params(z["params"])
        ws.xm, ws.xs, ws.tm, ws.ts = z["xm"], z["xs"], z["tm"], z["ts"]
        ws._push_normalization()
        return ws

    def step(self, ws: Workspace, opts: CoOpts, dopt, x, w, S0: float, dt: float, v_new,
             retry: bool = True, use_network: bool = True) -> dict:
        """One whole time step through co_step_learned_dev: the start with the
        smallest first residual among the learned proposal, the explicit
        predictor and the previous-step state, the implicit solve (dopt: defect
        correction; None: step_anderson!), one retry from the next start if it
        does not converge, and the entropy of the new state. x, w, v_new are
        torch CUDA tensors ((2, N), (N,), (2, N)); returns the step record."""
        from . import CoStepInfo
        info = CoStepInfo()
        N = x.shape[1]
        _check(ws.lib.co_step_learned_dev(ws.h, C.byref(opts),
                                          C.byref(dopt) if dopt is not None else None,
                                          self.mlp.h if use_network else None, int(retry),
                                          v_new.data_ptr(), x.data_ptr(), w.data_ptr(), N, S0, dt,
                                          C.byref(info)), "co_step_learned_dev")
        return info.as_dict()


def step_defect_warm(ws: Workspace, warm: "WarmStart", opts: CoOpts, dopt, x, w, S0: float,
                     dt: float, v1, retry: bool = True):
    """One implicit step from x (torch (2, N)) by defect correction from the
    learned warm start (WarmStart.step, i.e. co_step_learned_dev). v1 receives
    the new markers. Returns (outer, residual, inner, r0) and the step record."""
    rec = warm.step(ws, opts, dopt, x, w, S0, dt, v1, retry=retry)
    return (rec["outer"], rec["res"], rec["inner"], rec["r0"]), rec


def generate_pairs(ws: Workspace, opts: CoOpts, v, w, dt: float, steps: int, solve):
    """Run `steps` time steps from v (torch (2, N)); `solve(v1, v, S0)` performs
    the implicit step in place on v1 and returns True when it converged.
    Returns (X, T, x): features at each converged step's start and delta =
    (v_converged - v_pred)/dt^2 as numpy arrays (steps whose solve did not
    converge are advanced but not kept: their delta is not a fixed point), and
    the final state."""
    import torch
    Xs, Ts = [], []
    x = v.clone()
    for _ in range(steps):
        S0 = entropy_of(ws, x, w)
        X, vp, _rp = features(ws, opts, x, w, S0, dt)
        v1 = vp.clone()
        ok = solve(v1, x, S0)
        if ok is None or ok:
            delta = ((v1 - vp) / (dt * dt)).T.contiguous()
            Xs.append(X.cpu().numpy())
            Ts.append(delta.cpu().numpy())
        x = v1
    if not Xs:
        n = N_IN
        return np.zeros((0, n), np.float32), np.zeros((0, N_OUT), np.float32), x
    return np.concatenate(Xs), np.concatenate(Ts), x


def entropy_of(ws: Workspace, v, w) -> float:
    S = C.c_double()
    _check(ws.lib.co_entropy_of_markers_dev(ws.h, v.data_ptr(), w.data_ptr(), v.shape[1],
                                            C.byref(S)), "co_entropy_of_markers_dev")
    return S.value


__all__ = ["MLP", "WarmStart", "features", "generate_pairs", "entropy_of", "CollopsError"]
