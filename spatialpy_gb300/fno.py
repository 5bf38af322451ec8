"""Host side of the surrogate network's kernels (``csrc/fno.cu``; the
``sp_fno_*`` entry points of ``include/spgpu.h``).

``FnoNet`` owns one ``sp_fno`` handle: the fp32 parameters, their bf16 copy,
gradients, Adam moments and the activation workspace for ``max_batch``
samples live on the GPU.  Inputs and outputs are torch CUDA tensors (PyTorch
supplies device memory and the current stream); every computation is one of
this library's kernels.  The product path raises when ``libspgpu.so`` is
missing or the GPU is absent.

``param_layout`` is the flat parameter order the C ABI defines;
``init_params`` fills it the way the usual layer initialisers do (uniform
within 1/sqrt(fan_in) for the pointwise and dense layers, a normal of scale
1/width^2 for the spectral weights).
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from . import abi


@dataclasses.dataclass(frozen=True)
class FnoShape:
    n: int                  # lattice edge
    width: int = 32
    modes: int = 12
    layers: int = 4
    in_ch: int = 6
    out_ch: int = 6
    cond: int = 6
    hidden: int = 64
    max_batch: int = 64

    @property
    def num_modes(self) -> int:
        return 2 * self.modes * self.modes


def param_layout(s: FnoShape) -> dict:
    """name -> (offset, shape) in the flat parameter array (sp_fno_shape order)."""
    C_, M, H, G = s.width, s.num_modes, s.hidden, 2 * s.layers * s.width
    items = [("lift_w", (C_, s.in_ch)), ("lift_b", (C_,))]
    for k in range(s.layers):
        items += [(f"spec_w{k}", (M, C_, C_, 2)), (f"lin_w{k}", (C_, C_)), (f"lin_b{k}", (C_,))]
    items += [("film1_w", (H, s.cond)), ("film1_b", (H,)), ("film2_w", (G, H)), ("film2_b", (G,)),
              ("proj1_w", (H, C_)), ("proj1_b", (H,)), ("proj2_w", (s.out_ch, H)),
              ("proj2_b", (s.out_ch,))]
    out, off = {}, 0
    for name, shp in items:
        out[name] = (off, shp)
        off += int(np.prod(shp))
    out["_total"] = (off, ())
    return out


def num_params(s: FnoShape) -> int:
    return param_layout(s)["_total"][0]


def unpack(s: FnoShape, flat: np.ndarray) -> dict:
    """Views of the named parameter tensors in ``flat``."""
    out = {}
    for name, (off, shp) in param_layout(s).items():
        if name != "_total":
            out[name] = flat[off:off + int(np.prod(shp))].reshape(shp)
    return out


def init_params(s: FnoShape, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    flat = np.zeros(num_params(s), dtype=np.float32)
    P = unpack(s, flat)

    def uni(a, fan_in):
        bound = 1.0 / np.sqrt(fan_in)
        a[...] = rng.uniform(-bound, bound, a.shape)

    uni(P["lift_w"], s.in_ch); uni(P["lift_b"], s.in_ch)
    for k in range(s.layers):
        P[f"spec_w{k}"][...] = rng.standard_normal(P[f"spec_w{k}"].shape) / (s.width * s.width)
        uni(P[f"lin_w{k}"], s.width); uni(P[f"lin_b{k}"], s.width)
    uni(P["film1_w"], s.cond); uni(P["film1_b"], s.cond)
    uni(P["film2_w"], s.hidden); uni(P["film2_b"], s.hidden)
    uni(P["proj1_w"], s.width); uni(P["proj1_b"], s.width)
    uni(P["proj2_w"], s.hidden); uni(P["proj2_b"], s.hidden)
    return flat


def bf16_round(a: np.ndarray) -> np.ndarray:
    """fp32 values rounded to bf16 (nearest even), returned as fp32: the
    values the kernels compute with."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


class FnoError(RuntimeError):
    pass


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class FnoNet:
    """One network on the current CUDA device."""

    def __init__(self, shape: FnoShape, seed: int = 0, params: np.ndarray | None = None):
        import torch
        if not torch.cuda.is_available():
            raise FnoError("FnoNet needs a CUDA device")
        self.torch = torch
        self.shape = shape
        self.lib = abi.load_library()
        sh = abi.SpFnoShape(*(int(getattr(shape, f)) for f in
                              ("n", "width", "modes", "layers", "in_ch", "out_ch", "cond",
                               "hidden", "max_batch")))
        h = C.c_void_p()
        rc = self.lib.sp_fno_create(C.byref(sh), C.byref(h))
        if rc != 0:
            raise FnoError(f"sp_fno_create failed ({rc})")
        self.h = h
        self.count = int(self.lib.sp_fno_num_params(h))
        assert self.count == num_params(shape)
        self.set_params(init_params(shape, seed) if params is None else params)

    # -- plumbing -------------------------------------------------------
    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.lib.sp_fno_last_error(self.h).decode()
            raise FnoError(f"{what} failed ({rc}): {msg}")

    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def close(self):
        if getattr(self, "h", None):
            self.lib.sp_fno_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters -------------------------------------------------------
    def set_params(self, flat: np.ndarray):
        a = np.ascontiguousarray(flat, dtype=np.float32)
        self._check(self.lib.sp_fno_set_params(self.h, a.ctypes.data_as(C.POINTER(C.c_float)),
                                               a.size), "sp_fno_set_params")

    def get_params(self) -> np.ndarray:
        a = np.empty(self.count, dtype=np.float32)
        self._check(self.lib.sp_fno_get_params(self.h, a.ctypes.data_as(C.POINTER(C.c_float)),
                                               a.size), "sp_fno_get_params")
        return a

    def get_grads(self) -> np.ndarray:
        a = np.empty(self.count, dtype=np.float32)
        self._check(self.lib.sp_fno_get_grads(self.h, a.ctypes.data_as(C.POINTER(C.c_float)),
                                              a.size), "sp_fno_get_grads")
        return a

    # -- compute ----------------------------------------------------------
    def _field(self, t, ch, what):
        torch = self.torch
        if t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous():
            raise FnoError(f"{what}: contiguous float32 CUDA tensor required")
        if t.shape[-3:] != (ch, self.shape.n, self.shape.n) and t.shape[-2:] != (ch, self.shape.n ** 2):
            raise FnoError(f"{what}: shape {tuple(t.shape)} is not [.., {ch}, n, n]")

    def forward(self, x, cond, out=None):
        """x: [in_ch, n, n] shared by the batch, or [B, in_ch, n, n];
        cond [B, cond]; returns [B, out_ch, n, n]."""
        torch = self.torch
        s = self.shape
        B = cond.shape[0]
        if (cond.dtype != torch.float32 or not cond.is_cuda or not cond.is_contiguous()
                or cond.dim() != 2 or cond.shape[1] != s.cond):
            raise FnoError(f"cond: contiguous float32 CUDA tensor [B, {s.cond}] required")
        self._field(x, s.in_ch, "x")
        shared = 1 if x.dim() == 3 or (x.dim() == 4 and x.shape[0] == 1 and B > 1) else 0
        if not shared and x.shape[0] != B:
            raise FnoError("x and cond disagree on the batch size")
        if out is None:
            out = torch.empty(B, s.out_ch, s.n, s.n, dtype=torch.float32, device=cond.device)
        elif out.numel() != B * s.out_ch * s.n * s.n:
            raise FnoError("out: wrong size")
        self._field(out, s.out_ch, "out")
        # the backward pass reads x, cond and out of this call: keep them alive
        self._last = (x, cond, out)
        self._check(self.lib.sp_fno_forward(self.h, _ptr(x), shared, _ptr(cond), B, _ptr(out),
                                            self._stream()), "sp_fno_forward")
        return out

    def backward(self, target):
        """Gradients of the mean squared error of the last forward pass (whose
        x, cond and output tensors this object keeps alive)."""
        self._field(target, self.shape.out_ch, "target")
        self._check(self.lib.sp_fno_backward(self.h, _ptr(target), target.shape[0],
                                             self._stream()), "sp_fno_backward")

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        self._check(self.lib.sp_fno_adam(self.h, lr, beta1, beta2, eps, self._stream()),
                    "sp_fno_adam")

    def train_step(self, x, cond_all, target_all, idx: np.ndarray, lr: float,
                   beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        """One Adam step on the rows ``idx`` of (cond_all, target_all); x is
        shared ([in_ch, n, n]) or per row ([rows, in_ch, n, n])."""
        shared = 1 if x.dim() == 3 else 0
        rows = cond_all.shape[0]
        if target_all.shape[0] != rows or (not shared and x.shape[0] != rows):
            raise FnoError("train_step: cond, target and x disagree on the row count")
        ix = np.ascontiguousarray(idx, dtype=np.int32)
        self._check(self.lib.sp_fno_train_step(
            self.h, _ptr(x), shared, _ptr(cond_all), _ptr(target_all), cond_all.shape[0],
            ix.ctypes.data_as(C.POINTER(C.c_int32)), len(ix), lr, beta1, beta2, eps,
            self._stream()), "sp_fno_train_step")
        self._last = (x, cond_all, target_all)

    def loss(self) -> float:
        v = C.c_float()
        self._check(self.lib.sp_fno_loss(self.h, C.byref(v)), "sp_fno_loss")
        return float(v.value)
