"""Per-sample image comparison shared by the GPU parity tests.

Device and oracle renders of the same frame take the same random numbers, so their pixels agree to FP32 rounding
except where a rounding difference flips a branch of some path (Russian roulette, lobe choice, a hit on an edge).
`assert_match` requires a share of pixels within atol + rtol * |ref| on every channel, and reports the share it
measured and the worst pixel, so a failure shows what diverged. When the environment variable VKRT_PARITY_LOG names a
file, every comparison is appended to it as one JSON line (label, share, bound, worst pixel)."""
from __future__ import annotations

import json
import os

import numpy as np


def compare(gpu: np.ndarray, ref: np.ndarray, atol: float, rtol: float):
    """(share of pixels within tolerance on all RGB channels, worst pixel record, number of pixels outside)."""
    g = np.asarray(gpu, np.float64)[..., :3]
    r = np.asarray(ref, np.float64)[..., :3]
    err = np.abs(g - r)
    tol = atol + rtol * np.abs(r)
    ratio = (err / tol).max(-1)
    close = ratio <= 1.0
    k = np.unravel_index(int(np.argmax(ratio)), ratio.shape)
    worst = {"x": int(k[1]), "y": int(k[0]), "gpu": [round(v, 6) for v in g[k].tolist()],
             "ref": [round(v, 6) for v in r[k].tolist()], "err_over_tol": round(float(ratio[k]), 3)}
    return float(close.mean()), worst, int((~close).sum())


def assert_match(label: str | None, gpu: np.ndarray, ref: np.ndarray, atol: float, rtol: float,
                 max_outside: int) -> float:
    """At most `max_outside` pixels may differ by more than atol + rtol * |ref| on some channel; label None names
    the comparison after the running test."""
    if label is None:
        label = os.environ.get("PYTEST_CURRENT_TEST", "comparison").split(" ")[0]
    frac, worst, outside = compare(gpu, ref, atol, rtol)
    log = os.environ.get("VKRT_PARITY_LOG")
    if log:
        with open(log, "a") as f:
            f.write(json.dumps({"label": label, "share": frac, "outside": outside, "max_outside": max_outside,
                                "pixels": int(np.prod(np.shape(gpu)[:2])), "atol": atol, "rtol": rtol,
                                "worst": worst}) + "\n")
    assert outside <= max_outside, (f"{label}: {outside} pixels outside {atol} + {rtol}|ref| (at most {max_outside} "
                                    f"allowed; share within {frac:.5f}); worst {worst}")
    return frac


def relmse(x: np.ndarray, ref: np.ndarray) -> float:
    """Mean over pixels and channels of (x - ref)^2 / (ref^2 + 1e-2)."""
    x = np.asarray(x, np.float64)[..., :3]
    r = np.asarray(ref, np.float64)[..., :3]
    return float(np.mean((x - r) ** 2 / (r ** 2 + 1e-2)))
