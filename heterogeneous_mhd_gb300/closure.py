"""The learned closure: a periodic 3-D conv net on the coarse state, trained
and run by the BF16 tensor-core kernels of closure.cu (C ABI: mhd_closure.h).

Net: 8 input channels (rho, mx, my, mz, E, cell-centred Bx, By, Bz, each
standardised; padded to 16), four hidden 3^3 convolutions of 32 channels
with GELU, and a 1^3 head with 8 outputs: 5 fluid corrections and 3 edge
EMFs.  The correction of a coarse step is u += oscale * out[:5] and
b += bscale * (-curl E) with E = out[5:8] on the cell edges, so the B
correction is a constrained-transport update and leaves div B unchanged.

torch provides device memory and the stream; every operation on the data is
one of this package's kernels.  The reference has no learned closure.
"""
from __future__ import annotations

import ctypes as C
import json
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import MhdError, _check, lib

# kinds of mhd_cl_conv / mhd_cl_wgrad (include/mhd_closure.h)
FWD_IN, FWD_HID, FWD_HEAD, DGRAD_HEAD, DGRAD_HID = 0, 1, 2, 3, 4
WG_IN, WG_HID, WG_HEAD = 0, 1, 2

HIDDEN = 32
NLAYERS = 4  # hidden 3^3 layers


@dataclass(frozen=True)
class Layer:
    cout: int      # real output channels
    cin: int       # real input channels
    taps: int
    cout_pad: int  # packed layouts
    cin_pad: int
    dgrad: bool    # needs the flipped data-gradient weights

    @property
    def wsize(self) -> int:
        return self.cout * self.taps * self.cin


LAYERS = ([Layer(HIDDEN, 8, 27, HIDDEN, 16, False)] +
          [Layer(HIDDEN, HIDDEN, 27, HIDDEN, HIDDEN, True) for _ in range(NLAYERS - 1)] +
          [Layer(8, HIDDEN, 1, 16, HIDDEN, True)])


def _sig():
    L = lib()
    vp, i, ll, f, d = C.c_void_p, C.c_int, C.c_longlong, C.c_float, C.c_double
    sig = {
        "mhd_cl_conv": (i, [i, vp, vp, vp, vp, vp, vp, i, i, vp]),
        "mhd_cl_wgrad_scratch": (ll, [i, i, i]),
        "mhd_cl_wgrad": (i, [i, vp, vp, vp, vp, i, i, vp]),
        "mhd_cl_colsum": (i, [vp, i, ll, i, vp, vp, vp]),
        "mhd_cl_loss": (i, [vp, vp, vp, vp, vp, vp, i, i, vp]),
        "mhd_cl_features": (i, [vp, vp, i, vp, vp, vp, vp, vp]),
        "mhd_cl_normalize": (i, [vp, i, ll, vp, vp, vp, i, vp]),
        "mhd_cl_moments": (i, [vp, i, ll, vp, vp]),
        "mhd_cl_filter": (i, [vp, vp, i, i, vp, vp, vp]),
        "mhd_cl_diff": (i, [vp, vp, vp, vp, i, vp, vp]),
        "mhd_cl_apply": (i, [vp, vp, vp, i, vp, f, vp, vp, vp, vp, f, vp, vp, f, vp]),
        "mhd_cl_adamw": (i, [vp, vp, vp, vp, ll, i, f, f, f, f, f, vp]),
        "mhd_cl_pack": (i, [vp, i, i, i, i, i, vp, vp, vp]),
        "mhd_cl_use_tcgen05": (i, [i]),
        "mhd_cl_device_errors": (i, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


_L = None


def cl():
    global _L
    if _L is None:
        _L = _sig()
    return _L


def _p(t) -> int | None:
    return None if t is None else t.data_ptr()


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise MhdError(2, "the closure kernels need a CUDA GPU")
    return torch


def stream_ptr() -> int:
    torch = _torch()
    return torch.cuda.current_stream().cuda_stream


# ------------------------------------------------------------------ model

@dataclass
class Stats:
    """Standardisation of the inputs and scales of the outputs."""
    mean: np.ndarray = field(default_factory=lambda: np.zeros(8))
    inv_std: np.ndarray = field(default_factory=lambda: np.ones(8))
    oscale: np.ndarray = field(default_factory=lambda: np.ones(5))
    bscale: float = 1.0

    def to_json(self) -> dict:
        return {"mean": [float(x) for x in self.mean], "inv_std": [float(x) for x in self.inv_std],
                "oscale": [float(x) for x in self.oscale], "bscale": float(self.bscale)}

    @staticmethod
    def from_json(d: dict) -> "Stats":
        return Stats(np.asarray(d["mean"], dtype=np.float64), np.asarray(d["inv_std"], dtype=np.float64),
                     np.asarray(d["oscale"], dtype=np.float64), float(d["bscale"]))


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initial weights, zero biases, the head scaled down."""
    rng = np.random.Generator(np.random.PCG64(seed))
    parts = []
    for li, l in enumerate(LAYERS):
        std = np.sqrt(2.0 / (l.cin * l.taps))
        if li == len(LAYERS) - 1:
            std *= 0.1
        parts.append(rng.normal(0.0, std, size=l.wsize))
        parts.append(np.zeros(l.cout))
    return np.concatenate(parts).astype(np.float32)


def param_offsets():
    offs, o = [], 0
    for l in LAYERS:
        offs.append((o, o + l.wsize))
        o += l.wsize + l.cout
    return offs, o


def unflatten(flat: np.ndarray):
    """[(w (cout,k,k,k,cin), b)] views of a flat parameter vector (float64)."""
    offs, _ = param_offsets()
    out = []
    for l, (ow, ob) in zip(LAYERS, offs):
        k = round(l.taps ** (1 / 3))
        out.append((np.asarray(flat[ow:ob], dtype=np.float64).reshape(l.cout, k, k, k, l.cin),
                    np.asarray(flat[ob:ob + l.cout], dtype=np.float64)))
    return out


class ClosureNet:
    """Parameters, optimiser state and activations for batches of nb boxes of edge n."""

    def __init__(self, params: np.ndarray | None = None, stats: Stats | None = None, seed: int = 0):
        torch = _torch()
        self.torch = torch
        self.dev = torch.device("cuda")
        p = init_params(seed) if params is None else np.asarray(params, dtype=np.float32)
        _, total = param_offsets()
        if p.size != total:
            raise ValueError(f"expected {total} parameters, got {p.size}")
        self.p = torch.from_numpy(p.copy()).to(self.dev)
        self.g = torch.zeros_like(self.p)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.step_count = 0
        self.stats = stats or Stats()
        # scale of the applied correction chosen on validation runs (1 = as trained),
        # and per coarse edge where it was calibrated there
        self.gain = 1.0
        self.gain_by_edge: dict[int, float] = {}
        self.wf = [torch.empty(l.cout_pad * l.taps * l.cin_pad, dtype=torch.bfloat16, device=self.dev)
                   for l in LAYERS]
        self.wd = [torch.empty(l.cout_pad * l.taps * l.cin_pad, dtype=torch.bfloat16, device=self.dev)
                   if l.dgrad else None for l in LAYERS]
        self._shape = None
        self._stat_dev = None
        self.pack()

    # ---- weights
    def pack(self) -> None:
        offs, _ = param_offsets()
        s = stream_ptr()
        for l, (ow, _), wf, wd in zip(LAYERS, offs, self.wf, self.wd):
            _check(cl().mhd_cl_pack(self.p.data_ptr() + 4 * ow, l.cout, l.cin, l.taps, l.cout_pad, l.cin_pad,
                                    _p(wf), _p(wd), s), "mhd_cl_pack")

    def bias_ptr(self, li: int) -> int:
        offs, _ = param_offsets()
        return self.p.data_ptr() + 4 * offs[li][1]

    def params_numpy(self) -> np.ndarray:
        return self.p.cpu().numpy().copy()

    def grads_numpy(self) -> np.ndarray:
        return self.g.cpu().numpy().copy()

    # ---- buffers
    def ensure(self, nb: int, n: int) -> None:
        """Buffers for batches of nb boxes of edge n (kept per shape)."""
        if self._shape == (nb, n):
            return
        if not hasattr(self, "_bufs"):
            self._bufs = {}
        if (nb, n) not in self._bufs:
            torch = self.torch
            nv = nb * n ** 3
            bf = dict(dtype=torch.bfloat16, device=self.dev)
            ws = max(int(cl().mhd_cl_wgrad_scratch(k, nb, n)) for k in (WG_IN, WG_HID, WG_HEAD))
            if ws < 0:
                raise MhdError(1, f"box edge {n} is not supported by the closure kernels")
            self._bufs[(nb, n)] = dict(
                a=[torch.empty(nv * HIDDEN, **bf) for _ in range(NLAYERS)],
                z=[torch.empty(nv * HIDDEN, **bf) for _ in range(NLAYERS)],
                out=torch.empty(nv * 8, dtype=torch.float32, device=self.dev),
                dout=torch.empty(nv * 16, **bf),
                dz=[torch.empty(nv * HIDDEN, **bf) for _ in range(2)],
                rb=torch.empty(nv * 3, dtype=torch.float32, device=self.dev),
                lsc=torch.empty(512, dtype=torch.float32, device=self.dev),
                loss_dev=torch.zeros(1, dtype=torch.float32, device=self.dev),
                wsc=torch.empty(ws // 4 + 1, dtype=torch.float32, device=self.dev),
                csc=torch.empty(256 * HIDDEN, dtype=torch.float32, device=self.dev))
        for k, v in self._bufs[(nb, n)].items():
            setattr(self, k, v)
        self._shape = (nb, n)

    # ---- forward / backward
    def forward(self, x, nb: int, n: int):
        """x: BF16 [nb, n^3, 16] standardised features; returns the FP32 [nb, n^3, 8] output tensor."""
        self.ensure(nb, n)
        s = stream_ptr()
        L = cl()
        _check(L.mhd_cl_conv(FWD_IN, _p(x), _p(self.wf[0]), self.bias_ptr(0), _p(self.a[0]), _p(self.z[0]), None,
                             nb, n, s), "conv in")
        for li in range(1, NLAYERS):
            _check(L.mhd_cl_conv(FWD_HID, _p(self.a[li - 1]), _p(self.wf[li]), self.bias_ptr(li), _p(self.a[li]),
                                 _p(self.z[li]), None, nb, n, s), "conv hidden")
        _check(L.mhd_cl_conv(FWD_HEAD, _p(self.a[-1]), _p(self.wf[-1]), self.bias_ptr(NLAYERS), _p(self.out), None,
                             None, nb, n, s), "conv head")
        return self.out

    def loss(self, target, nb: int, n: int) -> None:
        """Loss of the last forward against BF16 [nb, n^3, 8] targets; fills dout; result via loss_value()."""
        _check(cl().mhd_cl_loss(_p(self.out), _p(target), _p(self.dout), _p(self.rb), _p(self.lsc),
                                _p(self.loss_dev), nb, n, stream_ptr()), "mhd_cl_loss")
        self._loss_norm = 8.0 * nb * n ** 3

    def loss_value(self) -> float:
        return float(self.loss_dev.item()) / self._loss_norm

    def backward(self, x, nb: int, n: int, dout=None) -> None:
        """Parameter gradients into self.g from d loss / d out (self.dout unless given)."""
        dout = self.dout if dout is None else dout
        s = stream_ptr()
        L = cl()
        offs, _ = param_offsets()
        gp = self.g.data_ptr()
        nv = nb * n ** 3
        # head
        _check(L.mhd_cl_wgrad(WG_HEAD, _p(self.a[-1]), _p(dout), _p(self.wsc), gp + 4 * offs[-1][0], nb, n, s),
               "wgrad head")
        _check(L.mhd_cl_colsum(_p(dout), 16, nv, 8, _p(self.csc), gp + 4 * offs[-1][1], s), "colsum head")
        cur = 0
        _check(L.mhd_cl_conv(DGRAD_HEAD, _p(dout), _p(self.wd[-1]), None, _p(self.dz[cur]), None, _p(self.z[-1]),
                             nb, n, s), "dgrad head")
        for li in range(NLAYERS - 1, 0, -1):
            dz = self.dz[cur]
            _check(L.mhd_cl_wgrad(WG_HID, _p(self.a[li - 1]), _p(dz), _p(self.wsc), gp + 4 * offs[li][0], nb, n,
                                  s), "wgrad hidden")
            _check(L.mhd_cl_colsum(_p(dz), HIDDEN, nv, HIDDEN, _p(self.csc), gp + 4 * offs[li][1], s),
                   "colsum hidden")
            _check(L.mhd_cl_conv(DGRAD_HID, _p(dz), _p(self.wd[li]), None, _p(self.dz[1 - cur]), None,
                                 _p(self.z[li - 1]), nb, n, s), "dgrad hidden")
            cur = 1 - cur
        dz = self.dz[cur]
        _check(L.mhd_cl_wgrad(WG_IN, _p(x), _p(dz), _p(self.wsc), gp + 4 * offs[0][0], nb, n, s), "wgrad in")
        _check(L.mhd_cl_colsum(_p(dz), HIDDEN, nv, HIDDEN, _p(self.csc), gp + 4 * offs[0][1], s), "colsum in")

    def adamw(self, lr: float, beta1=0.9, beta2=0.999, eps=1e-8, wd=1e-4) -> None:
        self.step_count += 1
        _check(cl().mhd_cl_adamw(_p(self.p), _p(self.g), _p(self.m), _p(self.v), self.p.numel(), self.step_count,
                                 lr, beta1, beta2, eps, wd, stream_ptr()), "mhd_cl_adamw")
        self.pack()

    # ---- inference on a coarse state
    def _stat_tensors(self):
        if self._stat_dev is None:
            t = self.torch
            st = self.stats
            self._stat_dev = (t.tensor(st.mean, dtype=t.float32, device=self.dev),
                              t.tensor(st.inv_std, dtype=t.float32, device=self.dev),
                              t.tensor(st.oscale, dtype=t.float32, device=self.dev))
        return self._stat_dev

    def features(self, u, b, n: int, x) -> None:
        mean, inv, _ = self._stat_tensors()
        _check(cl().mhd_cl_features(u, b, n, _p(mean), _p(inv), None, _p(x), stream_ptr()), "mhd_cl_features")

    # ---- persistence
    def save(self, path) -> None:
        path = Path(path)
        np.savez_compressed(path, params=self.params_numpy(),
                            meta=np.frombuffer(json.dumps({"stats": self.stats.to_json(),
                                                           "layers": [l.__dict__ for l in LAYERS],
                                                           "steps": self.step_count,
                                                           "gain": self.gain,
                                                           "gain_by_edge": {str(k): v for k, v in
                                                                            self.gain_by_edge.items()}}).encode(),
                                            dtype=np.uint8))

    @staticmethod
    def load(path) -> "ClosureNet":
        with np.load(path) as z:
            params = z["params"]
            meta = json.loads(bytes(z["meta"]).decode())
        net = ClosureNet(params, Stats.from_json(meta["stats"]))
        net.gain = float(meta.get("gain", 1.0))
        net.gain_by_edge = {int(k): float(v) for k, v in meta.get("gain_by_edge", {}).items()}
        return net

    def gain_for(self, n: int) -> float:
        """The calibrated correction gain for coarse boxes of edge n."""
        return self.gain_by_edge.get(int(n), self.gain)


class Corrector:
    """Applies a trained net to one coarse box after each plain step; `gain`
    scales the correction (1 = as trained; None = the net's calibrated gain)."""

    def __init__(self, net: ClosureNet, n: int, ecap: float = 1e-3, gain: float | None = None):
        t = net.torch
        gain = net.gain_for(n) if gain is None else gain
        self.net, self.n, self.ecap, self.gain = net, n, ecap, gain
        self.osc = t.tensor(np.asarray(net.stats.oscale) * gain, dtype=t.float32, device=net.dev)
        nv = n ** 3
        self.x = t.empty(nv * 16, dtype=t.bfloat16, device=net.dev)
        self.ut = t.empty(nv * 5, dtype=t.float32, device=net.dev)
        self.bt = t.empty(nv * 3, dtype=t.float32, device=net.dev)
        self.flags = t.zeros(4, dtype=t.int32, device=net.dev)
        self.esum = t.zeros(8, dtype=t.float64, device=net.dev)
        self.fallbacks = t.zeros(1, dtype=t.int64, device=net.dev)
        self.applied = 0

    def features(self, u_ptr: int, b_ptr: int) -> None:
        """Net input from the state at (u_ptr, b_ptr): the only read of the state."""
        self.net.features(u_ptr, b_ptr, self.n, self.x)

    def forward(self) -> None:
        self.net.forward(self.x, 1, self.n)

    def predict(self, u_ptr: int, b_ptr: int) -> None:
        self.features(u_ptr, b_ptr)
        self.forward()

    def apply(self, u_ptr: int, b_ptr: int, dt_ptr: int | None = None, dt_min: float = 0.0) -> None:
        """Correct the state in place with the last prediction (or fall back); with dt_ptr
        (the device dt of the step just taken) nothing happens when that step was empty."""
        _check(cl().mhd_cl_apply(u_ptr, b_ptr, _p(self.net.out), self.n, _p(self.osc),
                                 float(self.net.stats.bscale * self.gain),
                                 _p(self.ut), _p(self.bt), _p(self.flags), _p(self.esum), self.ecap,
                                 _p(self.fallbacks), dt_ptr, float(dt_min), stream_ptr()), "mhd_cl_apply")
        self.applied += 1

    def fallback_count(self) -> int:
        return int(self.fallbacks.item())
