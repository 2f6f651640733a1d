"""Learned warm start of the multigrid: the network and its training step.

The reference starts each solve from the previous step's potential
(solver/multigrid.py:464-467). The engine can instead start from the linear
extrapolation phi(n-1) + (phi(n-1) - phi(n-2)) and add a learned correction: a
small 3-D convolutional encoder-decoder predicts the next second difference of
the potential from the density and the potential history. The multigrid then
still iterates to the same residual, so the prediction only changes the
starting point, and a zero output is exactly the extrapolation. The network
runs on an R^3 grid (R = G/2): four levels R .. R/8 with 16-32-64-128 channels,
3x3x3 kernels, BF16 weights and activations with FP32 accumulation, forward and
backward passes in ``csrc/warmstart.cu`` on the tensor cores. This module owns a
``gc_ws`` network object: parameter initialisation, forward, backward (loss
0.5 mean (y - target)^2), Adam, and saving/loading the parameters.

Input channels (f16 [4][R^3]), _c the mean over 2x2x2 fine nodes, d the change
of the potential between solves and dd its change: log(1 + rho_c / mean rho_c),
phi_c / rms, d_c / rms(d_c), dd_c / rms(dd_c), all of the previous step.
Target: dd_c of this step / rms(dd_c of the previous step).
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import torch

from galaxy_collision_gb300 import _native

N_LAYERS = 11
N_FEATURES = 4
WEIGHTS_PATH = Path(__file__).resolve().parent / "warmstart_weights.npz"


def layer_table() -> list[tuple[int, int, int, int]]:
    """(cin, cout, level, relu) of each convolution, in parameter order."""
    L = _native.load()
    out = []
    for i in range(N_LAYERS):
        ci, co, lv, rl = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        L.gc_ws_layer_info(i, C.byref(ci), C.byref(co), C.byref(lv), C.byref(rl))
        out.append((ci.value, co.value, lv.value, rl.value))
    return out


def param_slices(layers=None) -> list[tuple[slice, slice]]:
    """(weight slice, bias slice) of each layer in the flat parameter vector."""
    layers = layers or layer_table()
    out, off = [], 0
    for ci, co, _, _ in layers:
        w = slice(off, off + 27 * co * ci)
        off = w.stop
        b = slice(off, off + co)
        off = b.stop
        out.append((w, b))
    return out


def init_params(seed: int = 0, layers=None) -> np.ndarray:
    """He-normal weights (fan-in 27*cin of the used input channels), zero biases;
    the output layer starts at zero so the untrained network predicts no second
    difference (the extrapolated warm start)."""
    layers = layers or layer_table()
    rng = np.random.default_rng(seed)
    sl = param_slices(layers)
    p = np.zeros(sl[-1][1].stop, np.float32)
    for i, ((ci, co, _, _), (ws, _)) in enumerate(zip(layers, sl)):
        fan_in = 27 * (N_FEATURES if i == 0 else ci)
        w = rng.normal(0.0, np.sqrt(2.0 / fan_in), size=(27, co, ci)).astype(np.float32)
        if i == 0:
            w[:, :, N_FEATURES:] = 0.0
        if i == len(layers) - 1:
            w[:] = 0.0
        p[ws] = w.ravel()
    return p


class WarmStartNet:
    """One ``gc_ws`` network on the current CUDA device."""

    def __init__(self, R: int, params: np.ndarray | None = None, seed: int = 0):
        self._lib = _native.lib()
        h = C.c_void_p()
        st = self._lib.gc_ws_create(C.byref(h), int(R))
        if st != _native.GC_OK:
            raise (ValueError if st == _native.GC_ERR_ARG else _native.GCError)(f"gc_ws_create(R={R}) failed ({st})")
        self._h = h
        self.R = int(R)
        n = C.c_int64()
        self._lib.gc_ws_num_params(h, C.byref(n))
        self.nparams = int(n.value)
        self.device = torch.device("cuda", torch.cuda.current_device())
        self._loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        self.y = torch.zeros((R, R, R), dtype=torch.float32, device=self.device)
        self.step = 0
        self.set_params(init_params(seed) if params is None else params)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                self._lib.gc_ws_destroy(self._h)
                self._h = None
        except Exception:  # pragma: no cover - interpreter shutdown
            pass

    def _call(self, name: str, *args) -> None:
        self._lib.gc_ws_set_stream(self._h, _native.current_stream_handle())
        st = getattr(self._lib, name)(self._h, *args)
        if st != _native.GC_OK:
            msg = self._lib.gc_ws_last_error(self._h)
            msg = msg.decode() if msg else ""
            raise (ValueError if st == _native.GC_ERR_ARG else _native.GCError)(f"{name}: {msg} ({st})")

    # -- parameters ---------------------------------------------------------------
    def set_params(self, params) -> None:
        p = torch.as_tensor(np.asarray(params, np.float32) if not torch.is_tensor(params) else params)
        p = p.to(device=self.device, dtype=torch.float32).contiguous()
        if p.numel() != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.numel()}")
        self._call("gc_ws_set_params", C.c_void_p(p.data_ptr()))
        torch.cuda.current_stream().synchronize()
        self.step = 0

    def params(self) -> torch.Tensor:
        out = torch.empty(self.nparams, dtype=torch.float32, device=self.device)
        self._call("gc_ws_get_params", C.c_void_p(out.data_ptr()))
        return out

    def grads(self) -> torch.Tensor:
        out = torch.empty(self.nparams, dtype=torch.float32, device=self.device)
        self._call("gc_ws_get_grads", C.c_void_p(out.data_ptr()))
        return out

    # -- passes -----------------------------------------------------------------------
    def forward(self, feat: torch.Tensor) -> torch.Tensor:
        """feat: f16 (4, R, R, R) on the device -> y (R, R, R) f32 (a view owned by the net)."""
        R = self.R
        if feat.dtype != torch.float16 or tuple(feat.shape) != (N_FEATURES, R, R, R) or not feat.is_contiguous():
            raise ValueError(f"feat must be a contiguous float16 tensor of shape ({N_FEATURES}, {R}, {R}, {R})")
        self._call("gc_ws_forward", C.c_void_p(feat.data_ptr()), C.c_void_p(self.y.data_ptr()))
        return self.y

    def backward(self, target: torch.Tensor) -> torch.Tensor:
        """Gradient of 0.5 mean((y - target)^2) for the last forward; returns the loss (device)."""
        R = self.R
        if target.dtype != torch.float16 or tuple(target.shape) != (R, R, R) or not target.is_contiguous():
            raise ValueError(f"target must be a contiguous float16 tensor of shape ({R}, {R}, {R})")
        self._call("gc_ws_backward", C.c_void_p(target.data_ptr()), C.c_void_p(self._loss.data_ptr()))
        return self._loss

    def adam_step(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        self.step += 1
        self._call("gc_ws_adam", C.c_float(lr), C.c_float(beta1), C.c_float(beta2), C.c_float(eps), int(self.step))

    def autotune(self, iters: int = 3) -> np.ndarray:
        """Time every feasible tile plan of each layer's three passes and keep the
        fastest (activations are overwritten). Returns the best milliseconds,
        shape (layers, 3): forward, data gradient, weight gradient."""
        ms = (C.c_float * (3 * N_LAYERS))()
        self._call("gc_ws_autotune", int(iters), C.cast(ms, C.c_void_p))
        return np.array(ms[:], dtype=np.float64).reshape(N_LAYERS, 3)

    def plans(self) -> list[list[tuple[int, ...]]]:
        """Plan per layer and pass: (planes, lines, taps per group/pass, CTAs, M tiles)."""
        out = []
        for layer in range(N_LAYERS):
            row = []
            for kind in range(3):
                v = (C.c_int * 5)()
                st = self._lib.gc_ws_plan_info(self._h, layer, kind, C.cast(v, C.c_void_p))
                row.append(tuple(v[:]) if st == _native.GC_OK else None)
            out.append(row)
        return out

    def status(self, clear: bool = True) -> int:
        f = C.c_uint32()
        self._call("gc_ws_status", C.byref(f), int(clear))
        return int(f.value)

    # -- persistence ------------------------------------------------------------------
    def save(self, path=WEIGHTS_PATH, **meta) -> Path:
        path = Path(path)
        np.savez(path, params=self.params().cpu().numpy(), R=self.R, **meta)
        return path

    @classmethod
    def load(cls, path=WEIGHTS_PATH, R: int | None = None) -> "WarmStartNet":
        with np.load(Path(path)) as z:
            params = z["params"]
            r = int(z["R"]) if R is None else int(R)
        return cls(r, params=params)


__all__ = ["WarmStartNet", "init_params", "layer_table", "param_slices", "WEIGHTS_PATH", "N_FEATURES"]


def _main(argv=None):
    """Time the network at R: forward, and forward + backward + Adam (random
    inputs and parameters); ``--iters 2`` is the small case profiled with ncu."""
    import argparse

    ap = argparse.ArgumentParser(description="time the warm-start network")
    ap.add_argument("--R", type=int, default=128)
    ap.add_argument("--iters", type=int, default=10)
    ap.add_argument("--autotune", action="store_true")
    args = ap.parse_args(argv)
    from galaxy_collision_gb300 import _build

    _build.build()
    R = args.R
    net = WarmStartNet(R, seed=1)
    if args.autotune:
        net.autotune()
    g = torch.Generator(device="cuda").manual_seed(0)
    feat = torch.randn((N_FEATURES, R, R, R), device="cuda", generator=g).half()
    tgt = (0.1 * torch.randn((R, R, R), device="cuda", generator=g)).half()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    net.forward(feat)
    net.backward(tgt)
    net.adam_step(1e-3)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.iters):
        net.forward(feat)
    e1.record()
    torch.cuda.synchronize()
    fwd = e0.elapsed_time(e1) / args.iters
    e0.record()
    for _ in range(args.iters):
        net.forward(feat)
        net.backward(tgt)
        net.adam_step(1e-3)
    e1.record()
    torch.cuda.synchronize()
    train = e0.elapsed_time(e1) / args.iters
    if net.status() != 0:
        raise RuntimeError("tensor-core completion timed out")
    print(f"R={R} forward {fwd:.3f} ms, forward+backward+Adam {train:.3f} ms", flush=True)


if __name__ == "__main__":
    _main()
