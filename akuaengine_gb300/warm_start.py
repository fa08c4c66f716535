"""Learned lambda warm start: the network handle, training-pair collection and training.

The network (C ABI `akua_mlp_*`, tensor-core kernels in csrc/mlp.cuh) predicts, from eight
features of a particle at the start of a step, the lambda that a long plain solve accumulates
over that step.  A solver with the network attached (`PBFSolver.set_warm_start`) uses the
prediction in its first Jacobi iteration and runs its remaining iterations unchanged; the plain
iterated solver stays the fallback (detach the network) and `PBFSolver.density_error` measures both.

Training pairs come from the solver itself: a "teacher" solver runs the scene with many
iterations (20 by default) and `capture_training` records, every few steps, the features at the
start of the step and the lambda the step accumulated.  Training runs the network's own forward
and backward kernels with Adam on the GPU; torch is used only to hold device buffers and to
shuffle and slice them.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._abi import MLP_NORM, MLP_PARAMS, check, load_library

PARAM_SHAPES = [("W1", (64, 8)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)),
                ("W3", (64, 64)), ("b3", (64,)), ("w4", (64,)), ("b4", (1,))]
FEATURE_NAMES = ["density_constraint", "neighbours_over_32", "lambda_denominator",
                 "lambda_iteration_1", "previous_lambda_sum", "grad_constraint_norm",
                 "grad_constraint_along_gravity", "speed"]


def init_params(seed: int = 0) -> np.ndarray:
    """Uniform(+-sqrt(6 / (fan_in + fan_out))) weights, zero biases, a small output layer."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in PARAM_SHAPES:
        if name.startswith("b"):
            parts.append(np.zeros(shape))
        elif name == "w4":
            parts.append(rng.uniform(-1, 1, shape) * np.sqrt(6.0 / 65.0) * 0.5)
        else:
            fan_out, fan_in = shape
            parts.append(rng.uniform(-1, 1, shape) * np.sqrt(6.0 / (fan_in + fan_out)))
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)


class LambdaNet:
    """The network on the current CUDA device."""

    def __init__(self, params: np.ndarray | None = None, seed: int = 0):
        self._lib = load_library()
        h = ctypes.c_void_p()
        check(self._lib.akua_mlp_create(ctypes.byref(h)), "akua_mlp_create")
        self._h = h
        self.norm = np.concatenate([np.zeros(8), np.ones(8), [1.0, 1.0]]).astype(np.float32)
        self.set_params(init_params(seed) if params is None else params)

    @property
    def handle(self):
        return self._h

    def set_params(self, params) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != MLP_PARAMS:
            raise ValueError("expected %d parameters" % MLP_PARAMS)
        check(self._lib.akua_mlp_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p), p.size),
              "akua_mlp_set_params")

    def params(self) -> np.ndarray:
        p = np.zeros(MLP_PARAMS, dtype=np.float32)
        check(self._lib.akua_mlp_get_params(self._h, p.ctypes.data_as(ctypes.c_void_p), p.size),
              "akua_mlp_get_params")
        return p

    def set_normalization(self, mean, inv_std, out_scale: float, blend: float = 1.0) -> None:
        norm = np.concatenate([np.asarray(mean, np.float32).reshape(8),
                               np.asarray(inv_std, np.float32).reshape(8),
                               [np.float32(out_scale), np.float32(blend)]]).astype(np.float32)
        check(self._lib.akua_mlp_set_normalization(self._h, norm.ctypes.data_as(ctypes.c_void_p),
                                                   MLP_NORM), "akua_mlp_set_normalization")
        self.norm = norm

    @property
    def out_scale(self) -> float:
        return float(self.norm[16])

    @property
    def blend(self) -> float:
        return float(self.norm[17])

    def set_blend(self, blend: float) -> None:
        """The lambda a step uses: lambda0 + blend * (estimate - lambda0)."""
        self.set_normalization(self.norm[:8], self.norm[8:16], self.out_scale, float(blend))

    def fit_normalization(self, features, targets) -> None:
        """Per-feature mean and 1/std, and the targets' standard deviation as output scale
        (blend 1)."""
        import torch

        f = features.double()
        mean = f.mean(0)
        std = f.std(0)
        inv = torch.where(std > 1e-30, 1.0 / std.clamp_min(1e-30), torch.ones_like(std))
        scale = float(targets.double().std())
        if not scale > 0:
            scale = 1.0
        self.set_normalization(mean.cpu().numpy(), inv.cpu().numpy(), scale)

    def forward(self, features, out=None, stream=None):
        import torch

        n = features.shape[0]
        if out is None:
            out = torch.empty(n, dtype=torch.float32, device=features.device)
        _check_tensor(features, (n, 8))
        _check_tensor(out, (n,))
        check(self._lib.akua_mlp_forward(self._h, _ptr(features), _ptr(out), n, _stream(stream)),
              "akua_mlp_forward")
        return out

    def gradient(self, features, targets, stream=None) -> tuple[np.ndarray, float]:
        n = features.shape[0]
        _check_tensor(features, (n, 8))
        _check_tensor(targets, (n,))
        g = np.zeros(MLP_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        check(self._lib.akua_mlp_gradient(self._h, _ptr(features), _ptr(targets), n,
                                          g.ctypes.data_as(ctypes.c_void_p), ctypes.byref(loss),
                                          _stream(stream)), "akua_mlp_gradient")
        return g, float(loss.value)

    def adam_step(self, features, targets, lr: float, stream=None) -> None:
        n = features.shape[0]
        check(self._lib.akua_mlp_adam_step(self._h, _ptr(features), _ptr(targets), n, float(lr),
                                           _stream(stream)), "akua_mlp_adam_step")

    def synchronize(self, stream=None) -> None:
        check(self._lib.akua_mlp_synchronize(self._h, _stream(stream)), "akua_mlp_synchronize")

    def save(self, path: str) -> None:
        np.savez(path, params=self.params(), norm=self.norm)

    @classmethod
    def load(cls, path: str) -> "LambdaNet":
        d = np.load(path)
        net = cls(params=d["params"])
        norm = d["norm"]
        net.set_normalization(norm[:8], norm[8:16], float(norm[16]), float(norm[17]))
        return net

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            rc = self._lib.akua_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()
            check(rc, "akua_mlp_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    if stream is None:
        return None
    return ctypes.c_void_p(int(getattr(stream, "cuda_stream", stream)))


def _check_tensor(t, shape):
    if (not t.is_cuda or not t.is_contiguous() or str(t.dtype) != "torch.float32"
            or tuple(t.shape) != tuple(shape)):
        raise ValueError("expected a contiguous CUDA float32 tensor of shape %s" % (shape,))


def collect_pairs(sc, cfg, corr, steps: int, capture_every: int, first_capture: int = 2,
                  teacher_iterations: int = 20, stream=None):
    """Steps scene `sc` with a `teacher_iterations` solver for `steps` steps and returns the
    (features [M, 8], targets [M]) pairs captured every `capture_every` steps from step
    `first_capture` on (the first steps have no previous lambda sum to report)."""
    import torch

    from .solver import PBFConfig, PBFSolver

    tcfg = PBFConfig(**{**cfg.__dict__, "solverIterations": int(teacher_iterations)})
    solver = PBFSolver(sc.n, tcfg, corr, stream=stream)
    solver.set_lambda_tracking(True)
    buf = torch.from_numpy(sc.particles.view(np.uint8).copy()).cuda()
    feats, targs = [], []
    try:
        for k in range(steps):
            if k >= first_capture and (k - first_capture) % capture_every == 0:
                f = torch.empty((sc.n, 8), dtype=torch.float32, device="cuda")
                t = torch.empty(sc.n, dtype=torch.float32, device="cuda")
                solver.capture_training(f, t)
                feats.append(f)
                targs.append(t)
            solver.step(buf, sc.dt, sc.box_min, sc.box_max)
        solver.synchronize()
    finally:
        solver.close()
    return torch.cat(feats), torch.cat(targs)


def train(net: LambdaNet, features, targets, epochs: int = 8, batch: int = 65536,
          lr: float = 2e-3, lr_final: float = 2e-4, seed: int = 0, stream=None) -> list[float]:
    """Adam over shuffled minibatches with a geometric learning-rate decay; returns the loss on
    the whole set after each epoch (one gradient pass)."""
    import torch

    n = features.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    per_epoch = max(1, (n + batch - 1) // batch)
    total = epochs * per_epoch
    losses = []
    k = 0
    for _ in range(epochs):
        perm = torch.randperm(n, generator=g).to(features.device)
        xf, yf = features[perm].contiguous(), targets[perm].contiguous()
        for b0 in range(0, n, batch):
            rate = lr * (lr_final / lr) ** (k / max(total - 1, 1))
            net.adam_step(xf[b0:b0 + batch], yf[b0:b0 + batch], rate, stream)
            k += 1
        net.synchronize(stream)
        losses.append(net.gradient(features, targets, stream)[1])
    return losses


def rollout_errors(sc, cfg, corr, iterations: int, net=None, steps: int = 60, stream=None):
    """Density-constraint errors [(max C, mean |C|) per step] of `steps` steps of scene `sc` with
    `iterations` Jacobi iterations, warm-started by `net` when given."""
    import torch

    from .solver import PBFSolver

    s = PBFSolver(sc.n, cfg, corr, stream=stream)
    s.set_solver_iterations(iterations)
    if net is not None:
        s.set_warm_start(net)
    buf = torch.from_numpy(sc.particles.view(np.uint8).copy()).cuda()
    errs = []
    try:
        for _ in range(steps):
            s.step(buf, sc.dt, sc.box_min, sc.box_max)
            errs.append(s.density_error())
    finally:
        s.close()
    return np.array(errs)


def calibrate_blend(net: LambdaNet, sc, cfg, corr, iterations: int,
                    blends=(0.0, 0.05, 0.1, 0.15, 0.2, 0.3, 0.4, 0.5), steps: int = 60,
                    stream=None, max_tolerance: float | None = None) -> dict:
    """Rolls `sc` out with each blend and sets the best one.  Errors per rollout: the per-step
    max density error and mean |C|, each averaged over the rollout.  Without `max_tolerance` the
    best blend has the lowest max error (mean |C| breaks ties).  With it, the best blend has the
    lowest mean |C| among those whose max error is at most (1 + max_tolerance) times blend 0's.
    Blend 0 is the plain solver, so in both cases the choice is no worse than plain on that
    rollout by those measures.  Returns {blend: (mean of max C, mean of mean |C|)}."""
    res = {}
    for g in sorted(set(float(b) for b in blends) | {0.0}):
        net.set_blend(g)
        e = rollout_errors(sc, cfg, corr, iterations, net, steps, stream)
        bad = not np.isfinite(e).all()
        res[g] = (float("inf"), float("inf")) if bad else (float(e[:, 0].mean()),
                                                           float(e[:, 1].mean()))
    if max_tolerance is None:
        best = min(res, key=lambda g: (res[g][0], res[g][1]))
    else:
        bound = (1.0 + max_tolerance) * res[0.0][0]
        best = min((g for g in res if res[g][0] <= bound), key=lambda g: (res[g][1], res[g][0]))
    net.set_blend(best)
    return res


def calibrate_equal_error(net: LambdaNet, scenes, corr, iterations: int, targets,
                          blends=(0.25, 0.5, 0.75, 1.0), steps: int = 60, stream=None):
    """Zero-tolerance calibration against a plain solver's max error on several scenes: rolls
    each (scene, config) of `scenes` out with each blend at `iterations` warm-started iterations
    and keeps the blends whose max density error (mean over the rollout of the per-step max) is at
    most that scene's entry of `targets` on every scene.  Sets and returns the one of them with the
    lowest mean |C| summed over the scenes, or None (blend left at 0) when none qualifies; also
    returns {blend: [(max C, mean |C|) per scene]}."""
    res = {}
    for g in blends:
        net.set_blend(float(g))
        per = []
        for sc, cfg in scenes:
            e = rollout_errors(sc, cfg, corr, iterations, net, steps, stream)
            per.append((float(e[:, 0].mean()), float(e[:, 1].mean()))
                       if np.isfinite(e).all() else (float("inf"), float("inf")))
        res[float(g)] = per
    ok = [g for g in res if all(m <= t for (m, _), t in zip(res[g], targets))]
    best = min(ok, key=lambda g: sum(v[1] for v in res[g])) if ok else None
    net.set_blend(best if best is not None else 0.0)
    return best, res


def collect_mixed(scenes, corr, teacher_iterations: int, stream=None, collect=None):
    """Training pairs from several scenes: `scenes` is a list of (scene, config) (each config
    carries its scene's gravity); pairs of all scenes concatenated."""
    import torch

    collect = collect or {"steps": 90, "capture_every": 3, "first_capture": 2}
    xs, ys = [], []
    for sc, cfg in scenes:
        x, y = collect_pairs(sc, cfg, corr, teacher_iterations=teacher_iterations, stream=stream,
                             **collect)
        xs.append(x)
        ys.append(y)
    return torch.cat(xs), torch.cat(ys)


def fewest_iterations_at_equal_error(train_scenes, corr, *, calibration_scenes=None,
                                     plain_iterations: int = 4, candidates=(1, 2, 3),
                                     steps: int = 60, stream=None, collect=None, epochs: int = 6,
                                     batch: int = 65536, blends=(0.25, 0.5, 0.75, 1.0),
                                     seed: int = 0, keep_last: bool = False):
    """The learned warm start at equal max error.  `train_scenes` and `calibration_scenes`: lists
    of (scene, config) (calibration defaults to the training scenes).  For k = candidates in
    increasing order, trains a network whose target is the lambda sum of a
    (plain_iterations - k + 1)-iteration teacher (the learned first iteration stands in for the
    plain iterations it saves) on pairs from every training scene, calibrates its blend with zero
    tolerance against the plain solver's max error on every calibration scene, and stops at the
    first k that reaches it.  Returns (k, net or None, report); k = plain_iterations and no
    network when no candidate qualifies (with `keep_last`, the last candidate's network, blend set
    to the blend with the lowest worst-scene max error, is returned as report["last"])."""
    cal = calibration_scenes or train_scenes
    targets, plain_means = [], []
    for sc, cfg in cal:
        plain = rollout_errors(sc, cfg, corr, plain_iterations, None, steps, stream)
        targets.append(float(plain[:, 0].mean()))
        plain_means.append(float(plain[:, 1].mean()))
    report = {"plain_max": targets, "plain_mean_abs": plain_means, "tried": {}}
    ks = sorted(candidates)
    for k in ks:
        teacher = plain_iterations - k + 1
        x, y = collect_mixed(train_scenes, corr, teacher, stream, collect)
        net = LambdaNet(seed=seed)
        net.fit_normalization(x, y)
        train(net, x, y, epochs=epochs, batch=batch, stream=stream)
        pairs = int(x.shape[0])
        del x, y
        best, res = calibrate_equal_error(net, cal, corr, k, targets, blends, steps, stream)
        report["tried"][str(k)] = {"teacher_iterations": teacher, "blend": best, "pairs": pairs,
                                   "blends": {str(g): [[round(a, 5), round(b, 5)] for a, b in v]
                                              for g, v in res.items()}}
        if best is not None:
            return k, net, report
        if keep_last and k == ks[-1]:
            net.set_blend(min(res, key=lambda g: max(m / t for (m, _), t in zip(res[g], targets))))
            report["last"] = (k, net)
        else:
            net.close()
    return plain_iterations, None, report
