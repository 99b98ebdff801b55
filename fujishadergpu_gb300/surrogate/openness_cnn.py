"""A small convolutional surrogate of exact openness, trained on the GPU from
labels of the exact ray-march kernel (``fsg_openness``).

No counterpart in the reference, which runs the exact ray-march only
(algorithms/_impl_openness.py:31-132).  The network maps three per-pixel
channels -- the window's elevation relative to its mean in pixel units (so
that elevation differences over pixel distances give the slope ratios the
openness angles are made of), and the NaN-filled gradient dz/dx, dz/dy of the
stencil kernel -- to the directional mean angle in degrees.  Eight 3x3
convolutions of 32 channels with dilations 1, 2, ..., 128 (receptive field
511 px, enough for rays of 256 px), residual from the second layer on, ReLU,
and a 1x1 head: about 66k parameters.  Every convolution runs in the
implicit-GEMM tensor-core kernels of csrc/fsg_conv.cu (BF16 operands, FP32
accumulation), forward and backward; PyTorch holds the tensors and runs the
optimiser (AdamW) and the elementwise glue.

The exact kernel stays the arbiter: ``check_and_fallback`` recomputes a sampled
block of each tile exactly and redoes the whole tile exactly when the
surrogate's mean absolute error there exceeds the threshold (2 degrees).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .. import _arrays
from .. import _native as N

CH = 32
DILATIONS = (1, 2, 4, 8, 16, 32, 64, 128)
IN_CH = 3          # relative elevation (pixel units / 64), dz/dx, dz/dy
IN_PAD = 16        # input channels as stored (zero padded for the 16-wide MMA K slice)
ELEV_SCALE = 64.0  # relative elevation in pixel units is divided by this
ANGLE_SCALE = 90.0  # the network predicts degrees / 90


def _stream():
    return C.c_void_p(_arrays.current_stream_handle())


def _torch():
    import torch
    return torch


def surrogate_features(dem, *, pixel_size: float = 1.0, pixel_scale_x=None, pixel_scale_y=None):
    """Input channels [1][H][W][16] (float32) of one window (NaN = NoData -> zeros)."""
    torch = _torch()
    from ..algorithms._stencil import stencil_block
    v = _arrays.as_device_f32_2d(dem)
    z = v.tensor
    g = stencil_block(z, ["dx", "dy"], pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                      pixel_scale_y=pixel_scale_y)
    valid = torch.isfinite(z)
    zm = z[valid].mean() if bool(valid.any()) else torch.zeros((), device=z.device)
    px = float(pixel_size) if pixel_size else 1.0
    feat = torch.zeros((1, v.h, v.w, IN_PAD), device=z.device, dtype=torch.float32)
    feat[0, :, :, 0] = torch.where(valid, (z - zm) / (px * ELEV_SCALE), torch.zeros_like(z))
    feat[0, :, :, 1] = torch.nan_to_num(g["dx"], nan=0.0)
    feat[0, :, :, 2] = torch.nan_to_num(g["dy"], nan=0.0)
    return feat


# ------------------------------------------------------------ autograd glue
def _pack(w, cin, transpose=False):
    torch = _torch()
    kc = 1 if cin <= 16 else 2
    wb = torch.empty(9 * kc * 256, dtype=torch.int32, device=w.device)
    N.check(N.lib().fsg_conv_pack_weights(C.c_void_p(w.data_ptr()), cin, 1 if transpose else 0,
                                          C.c_void_p(wb.data_ptr()), _stream()))
    return wb


def _conv(x, wb, cin_pad, dil, bias=None, relu=False, flip=False, res=None):
    torch = _torch()
    B, H, W, _ = x.shape
    y = torch.empty((B, H, W, CH), device=x.device, dtype=torch.float32)
    N.check(N.lib().fsg_conv3x3(C.c_void_p(x.data_ptr()), cin_pad, B, H, W, dil, C.c_void_p(wb.data_ptr()),
                                C.c_void_p(bias.data_ptr() if bias is not None else 0), 1 if relu else 0,
                                1 if flip else 0, C.c_void_p(res.data_ptr() if res is not None else 0),
                                C.c_void_p(y.data_ptr()), _stream()))
    return y


def _make_fns():
    torch = _torch()

    class Conv3x3Relu(torch.autograd.Function):
        """h = relu(conv3x3_dil(x) + b) on the tensor-core kernels."""

        @staticmethod
        def forward(ctx, x, w, b, cin, dil):
            x = x.contiguous()
            cin_pad = x.shape[-1]
            h = _conv(x, _pack(w.detach(), cin), cin_pad, dil, bias=b.detach(), relu=True)
            ctx.save_for_backward(x, w, h)
            ctx.cin, ctx.dil = cin, dil
            return h

        @staticmethod
        def backward(ctx, gh):
            x, w, h = ctx.saved_tensors
            gz = (gh * (h > 0)).contiguous()
            B, H, W, cin_pad = x.shape
            gw = torch.zeros_like(w)
            N.check(N.lib().fsg_conv3x3_wgrad(C.c_void_p(x.data_ptr()), ctx.cin, cin_pad, B, H, W, ctx.dil,
                                              C.c_void_p(gz.data_ptr()), C.c_void_p(gw.data_ptr()), _stream()))
            gb = gz.sum(dim=(0, 1, 2))
            gx = None
            if ctx.needs_input_grad[0] and ctx.cin == CH:
                gx = _conv(gz, _pack(w.detach(), CH, transpose=True), CH, ctx.dil, flip=True)
            return gx, gw, gb, None, None

    class Head(torch.autograd.Function):
        @staticmethod
        def forward(ctx, h, w, b):
            h = h.contiguous()
            n = h.numel() // CH
            out = torch.empty(h.shape[:-1], device=h.device, dtype=torch.float32)
            N.check(N.lib().fsg_head_forward(C.c_void_p(h.data_ptr()), C.c_void_p(w.data_ptr()),
                                             C.c_float(float(b.item())), n, C.c_void_p(out.data_ptr()), _stream()))
            ctx.save_for_backward(h, w)
            return out

        @staticmethod
        def backward(ctx, go):
            h, w = ctx.saved_tensors
            go = go.contiguous()
            n = h.numel() // CH
            gh = torch.empty_like(h)
            gw = torch.zeros_like(w)
            gb = torch.zeros(1, device=h.device, dtype=torch.float32)
            N.check(N.lib().fsg_head_backward(C.c_void_p(h.data_ptr()), C.c_void_p(w.data_ptr()),
                                              C.c_void_p(go.data_ptr()), None, n, C.c_void_p(gh.data_ptr()),
                                              C.c_void_p(gw.data_ptr()), C.c_void_p(gb.data_ptr()), _stream()))
            return gh, gw, gb

    return Conv3x3Relu, Head


_FNS = None


def _fns():
    global _FNS
    if _FNS is None:
        _FNS = _make_fns()
    return _FNS


class OpennessSurrogate:
    """The surrogate network: FP32 master weights (BF16 in the kernels)."""

    def __init__(self, seed: int = 0, device: str = "cuda"):
        torch = _torch()
        gen = torch.Generator(device="cpu").manual_seed(seed)
        self.params: List = []
        self.layers = []
        for i, dil in enumerate(DILATIONS):
            cin = IN_CH if i == 0 else CH
            std = math.sqrt(2.0 / (9 * cin)) * (1.0 if i == 0 else 0.5)
            w = (torch.randn(9, cin, CH, generator=gen) * std).to(device).requires_grad_()
            b = torch.zeros(CH, device=device).requires_grad_()
            self.layers.append((w, b, cin, dil))
            self.params += [w, b]
        self.head_w = (torch.randn(CH, generator=gen) * 0.05).to(device).requires_grad_()
        self.head_b = torch.full((1,), 0.5, device=device).requires_grad_()
        self.params += [self.head_w, self.head_b]

    def n_params(self) -> int:
        return int(sum(p.numel() for p in self.params))

    def forward(self, feat):
        """feat [B][H][W][16] -> predicted mean angle / 90, [B][H][W]."""
        Conv, Head = _fns()
        x = feat
        for i, (w, b, cin, dil) in enumerate(self.layers):
            h = Conv.apply(x, w, b, cin, dil)
            x = h if i == 0 else x + h
        return Head.apply(x, self.head_w, self.head_b)

    def predict_degrees(self, dem, *, pixel_size=1.0, pixel_scale_x=None, pixel_scale_y=None):
        """Mean openness angle in degrees of one window (NaN at NoData)."""
        torch = _torch()
        v = _arrays.as_device_f32_2d(dem)
        with torch.no_grad():
            w16 = ((v.w + 15) // 16) * 16
            z = v.tensor
            if w16 != v.w:  # the conv kernels take widths in multiples of 16: pad with NoData
                z = torch.nn.functional.pad(z, (0, w16 - v.w), value=float("nan"))
            feat = surrogate_features(z, pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                                      pixel_scale_y=pixel_scale_y)
            out = self.forward(feat)[0, :, :v.w] * ANGLE_SCALE
            return torch.where(torch.isfinite(v.tensor), out, torch.full_like(out, float("nan")))

    # ------------------------------------------------------------- persistence
    def state(self) -> Dict[str, np.ndarray]:
        d = {}
        for i, (w, b, cin, dil) in enumerate(self.layers):
            d[f"w{i}"] = w.detach().cpu().numpy()
            d[f"b{i}"] = b.detach().cpu().numpy()
        d["head_w"] = self.head_w.detach().cpu().numpy()
        d["head_b"] = self.head_b.detach().cpu().numpy()
        return d

    def load(self, d: Dict[str, np.ndarray]):
        torch = _torch()
        with torch.no_grad():
            for i, (w, b, cin, dil) in enumerate(self.layers):
                w.copy_(torch.from_numpy(np.asarray(d[f"w{i}"])))
                b.copy_(torch.from_numpy(np.asarray(d[f"b{i}"])))
            self.head_w.copy_(torch.from_numpy(np.asarray(d["head_w"])))
            self.head_b.copy_(torch.from_numpy(np.asarray(d["head_b"])))
        return self


# ------------------------------------------------------------------ training
def exact_degrees(dem, *, max_distance=256, num_directions=16, pixel_size=5.0, openness_type="positive"):
    from ..algorithms._impl_openness import compute_openness_raw_degrees
    return compute_openness_raw_degrees(dem, openness_type=openness_type, num_directions=num_directions,
                                        max_distance=max_distance, pixel_size=pixel_size)


def training_windows(n: int, size: int, *, seed: int = 0, pixel_size: float = 5.0, max_distance: int = 256):
    """Seeded synthetic fBm + ridged DEM windows with their exact labels (degrees)."""
    from .. import synth
    out = []
    for i in range(n):
        dem = synth.fbm_ridged_device(size, size, hurst=0.6 + 0.3 * ((i * 7919) % 100) / 100.0,
                                      seed_fbm=seed + 2 * i, seed_ridged=seed + 2 * i + 1, lo=0.0,
                                      hi=500.0 + 3500.0 * ((i * 104729) % 97) / 97.0)
        lab = exact_degrees(dem, max_distance=max_distance, pixel_size=pixel_size)
        out.append((surrogate_features(dem, pixel_size=pixel_size)[0], lab))
    return out


def train(model: OpennessSurrogate, windows, *, steps: int = 300, batch: int = 4, lr: float = 1e-3,
          margin: int = 256, seed: int = 0, log=None):
    """AdamW on the L1 loss (degrees) over the windows' interiors (pixels whose rays stay inside)."""
    torch = _torch()
    opt = torch.optim.AdamW(model.params, lr=lr, weight_decay=1e-4)
    rng = np.random.default_rng(seed)
    feats = torch.stack([f for f, _ in windows])
    labs = torch.stack([l for _, l in windows]) / ANGLE_SCALE
    sl = (slice(None), slice(margin, -margin), slice(margin, -margin))
    hist = []
    for step in range(steps):
        for gp in opt.param_groups:  # cosine decay to 5 % of the initial rate
            gp["lr"] = lr * (0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * step / max(1, steps))))
        idx = torch.from_numpy(rng.choice(len(windows), size=min(batch, len(windows)), replace=False))
        x = feats[idx.to(feats.device)]
        y = labs[idx.to(labs.device)]
        pred = model.forward(x)
        m = torch.isfinite(y[sl])
        loss = (pred[sl][m] - y[sl][m]).abs().mean()
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        hist.append(float(loss.item()) * ANGLE_SCALE)
        if log and (step % 50 == 0 or step == steps - 1):
            log(step, hist[-1])
    return hist


def mae_degrees(model: OpennessSurrogate, dem, label, *, pixel_size=5.0, margin=256) -> float:
    torch = _torch()
    pred = model.predict_degrees(dem, pixel_size=pixel_size)
    sl = (slice(margin, -margin), slice(margin, -margin))
    d = (pred[sl] - label[sl]).abs()
    return float(d[torch.isfinite(d)].mean().item())


# ------------------------------------------------------------ the tile loop
def load_default(device: str = "cuda") -> Optional[OpennessSurrogate]:
    """The surrogate trained by ``train.py`` (committed weights), or None if absent."""
    import os
    p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "openness_r256.npz")
    if not os.path.exists(p):
        return None
    with np.load(p) as d:
        return OpennessSurrogate(seed=0, device=device).load({k: d[k] for k in d.files})


def surrogate_tile_loop(dem, infos, model: OpennessSurrogate, *, pixel_size: float = 5.0, max_distance: int = 256,
                        num_directions: int = 16, threshold_deg: float = 2.0, check: int = 128,
                        out=None) -> Dict[str, object]:
    """Mean openness angle (degrees) of every tile core from the surrogate, checked against the exact
    kernel: an exact check block of ``check`` x ``check`` pixels at each core's centre; a tile
    whose block MAE exceeds ``threshold_deg`` is recomputed exactly.  ``infos``: TileInfo list
    (windows with a halo >= max_distance).  Returns the plane and the per-tile report."""
    torch = _torch()
    from ..algorithms import _impl_openness as OP
    v = _arrays.as_device_f32_2d(dem)
    plane = out if out is not None else torch.full((v.h, v.w), float("nan"), device=v.tensor.device)
    params = OP.make_params(openness_type="positive", num_directions=num_directions, max_distance=max_distance,
                            pixel_size=pixel_size)
    report = {"tiles": 0, "exact_redone": 0, "check_mae_deg": []}
    for t in infos:
        win = v.tensor[t.win_y:t.win_y + t.win_h, t.win_x:t.win_x + t.win_w]
        pred = model.predict_degrees(win, pixel_size=pixel_size)
        cy, cx = t.core_y - t.win_y, t.core_x - t.win_x
        core = pred[cy:cy + t.core_h, cx:cx + t.core_w]
        # exact check block at the core centre
        bh, bw = min(check, t.core_h), min(check, t.core_w)
        by = t.core_y + (t.core_h - bh) // 2
        bx = t.core_x + (t.core_w - bw) // 2
        tile = N.Tile()
        tile.win_y0, tile.win_x0, tile.win_h, tile.win_w = t.win_y, t.win_x, t.win_h, t.win_w
        tile.core_y0, tile.core_x0, tile.core_h, tile.core_w = by, bx, bh, bw
        tile.out_y0, tile.out_x0 = 0, 0
        tile.pixel_scale_x, tile.pixel_scale_y = pixel_size, -pixel_size
        ex = torch.empty((bh, bw), device=v.tensor.device)
        OP.run_openness(v, [tile], params, None, ex)
        blk = core[by - t.core_y:by - t.core_y + bh, bx - t.core_x:bx - t.core_x + bw]
        d = (blk - ex).abs()
        d = d[torch.isfinite(d)]
        mae = float(d.mean().item()) if d.numel() else 0.0
        report["tiles"] += 1
        report["check_mae_deg"].append(round(mae, 4))
        dst = plane[t.core_y:t.core_y + t.core_h, t.core_x:t.core_x + t.core_w]
        if mae > threshold_deg:
            report["exact_redone"] += 1
            tile.core_y0, tile.core_x0, tile.core_h, tile.core_w = t.core_y, t.core_x, t.core_h, t.core_w
            OP.run_openness(v, [tile], params, None, dst)
        else:
            dst.copy_(core)
    report["plane"] = plane
    return report
