"""Train the openness surrogate on the GPU from exact-kernel labels.

    python -m fujishadergpu_gb300.surrogate.train --windows 48 --size 1024 --steps 600 \
        --out fujishadergpu_gb300/surrogate/openness_r256.npz

Windows are seeded synthetic fBm + ridged DEMs at 5 m; labels are the exact
ray-march (reference sampling, 16 directions, R = 256) of each window; the
loss (L1, degrees) covers the pixels whose rays stay inside the window.
Prints one JSON line: training time, loss history endpoints, held-out MAE.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--windows", type=int, default=48)
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--max-distance", type=int, default=256)
    ap.add_argument("--holdout", type=int, default=4)
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    import torch
    from . import openness_cnn as S
    t0 = time.perf_counter()
    wins = S.training_windows(a.windows, a.size, seed=a.seed, pixel_size=5.0, max_distance=a.max_distance)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    model = S.OpennessSurrogate(seed=a.seed)
    t0 = time.perf_counter()
    hist = S.train(model, wins, steps=a.steps, batch=a.batch, lr=a.lr, margin=a.max_distance, seed=a.seed)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del wins
    from .. import synth
    maes = []
    for i in range(a.holdout):
        dem = synth.fbm_ridged_device(a.size, a.size, hurst=0.65 + 0.05 * i, seed_fbm=a.seed + 10_000 + 2 * i,
                                      seed_ridged=a.seed + 10_001 + 2 * i, lo=0.0, hi=1000.0 + 800.0 * i)
        lab = S.exact_degrees(dem, max_distance=a.max_distance, pixel_size=5.0)
        maes.append(S.mae_degrees(model, dem, lab, pixel_size=5.0, margin=a.max_distance))
    if a.out:
        np.savez_compressed(a.out, **model.state())
    print(json.dumps({"params": model.n_params(), "windows": a.windows, "size": a.size, "steps": a.steps,
                      "data_s": round(t_data, 2), "train_s": round(t_train, 2),
                      "loss_start_deg": round(float(np.mean(hist[:5])), 3),
                      "loss_end_deg": round(float(np.mean(hist[-20:])), 3),
                      "holdout_mae_deg": [round(m, 3) for m in maes]}))


if __name__ == "__main__":
    main()
