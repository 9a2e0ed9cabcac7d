"""Autotuner for the batched persistent factor + solve (ooc_batched_dposv / _sposv).

The kernel's per-matrix panel width is the tuning knob: wide panels put more of the flops
in the register-tiled trailing update (fewer passes over the trailing matrix), narrow ones
shorten the serial diagonal-block and row-solve steps for small orders.  For each size bucket (n in [32 q, 32 q + 31]) the
tuner times every candidate width on a synthetic batch of that bucket (A = M M^T / n + I,
M ~ N(0, 1)), keeps the fastest, and persists the 16-entry table as JSON keyed by GPU
name and precision:

    python -m oocdag_gb300.autotune [--prec fp64|fp32] [--out PATH]

``load_table`` returns the cached table (or None), which ``Handle.batched_posv`` takes as
``blk_table``.
"""
from __future__ import annotations

import argparse
import json
import os
import time

NBUCKETS = 16
CANDIDATES = {"fp64": (8, 16, 32), "fp32": (16, 32)}


def default_path() -> str:
    base = os.environ.get("OOC_AUTOTUNE_DIR") or os.path.join(os.path.expanduser("~"), ".cache", "oocdag_gb300")
    return os.path.join(base, "batched_autotune.json")


def _gpu_name() -> str:
    import torch

    return torch.cuda.get_device_name(0)


def make_batch(ns, seed: int, dtype, device="cuda"):
    """A_i = M M^T / n + I (M ~ N(0,1)), b_i ~ N(0,1), packed column-major on the device."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    a_off, b_off, As, Bs = [], [], [], []
    ao = bo = 0
    for n in ns:
        n = int(n)
        M = torch.randn((n, n), dtype=torch.float64, device=device, generator=g)
        A = M @ M.T / n + torch.eye(n, dtype=torch.float64, device=device)
        As.append(A.T.contiguous().reshape(-1))  # column-major storage of a symmetric matrix
        Bs.append(torch.randn(n, dtype=torch.float64, device=device, generator=g))
        a_off.append(ao)
        b_off.append(bo)
        ao += n * n
        bo += n
    tdt = torch.float64 if dtype == "fp64" else torch.float32
    return torch.cat(As).to(tdt), torch.cat(Bs).to(tdt), a_off, b_off


def tune(handle, prec: str = "fp64", flops_per_bucket: float = 4e9, reps: int = 2, seed: int = 0) -> dict:
    import numpy as np

    rng = np.random.default_rng(seed)
    table, timings = [], {}
    for q in range(NBUCKETS):
        lo, hi = max(1, 32 * q), 32 * q + 31
        mean_n = (lo + hi) / 2
        count = int(min(4000, max(64, flops_per_bucket / (mean_n ** 3 / 3))))
        ns = [int(x) for x in rng.integers(lo, hi + 1, size=count)]
        A0, B0, a_off, b_off = make_batch(ns, seed + q, prec)
        best, best_t = None, None
        timings[q] = {}
        for blk in CANDIDATES[prec]:
            ts = []
            for _ in range(reps):
                A = A0.clone()
                B = B0.clone()
                info, sec = handle.batched_posv(prec, ns, a_off, b_off, A, B, blk_table=[blk] * NBUCKETS)
                if any(info):
                    bad = [(ns[i], info[i]) for i in range(len(ns)) if info[i]][:5]
                    raise RuntimeError(f"batched {prec} blk={blk} bucket {q}: info != 0 for (n, info) {bad}")
                ts.append(sec)
            t = min(ts)
            timings[q][blk] = t
            if best_t is None or t < best_t:
                best, best_t = blk, t
        table.append(best)
    return {"gpu": _gpu_name(), "prec": prec, "table": table, "timings_s": timings, "when": time.time(),
            "candidates": list(CANDIDATES[prec])}


def save(result: dict, path: str | None = None) -> str:
    path = path or default_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    data = {}
    if os.path.exists(path):
        try:
            data = json.load(open(path))
        except Exception:
            data = {}
    data[f"{result['gpu']}|{result['prec']}"] = result
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1)
    os.replace(tmp, path)
    return path


def load_table(prec: str, path: str | None = None) -> list[int] | None:
    path = path or default_path()
    if not os.path.exists(path):
        return None
    try:
        data = json.load(open(path))
        return data[f"{_gpu_name()}|{prec}"]["table"]
    except Exception:
        return None


def main() -> None:
    import oocdag_gb300 as ooc

    p = argparse.ArgumentParser()
    p.add_argument("--prec", default="fp64", choices=["fp64", "fp32"])
    p.add_argument("--out", default=None)
    args = p.parse_args()
    with ooc.Handle(0) as h:
        res = tune(h, args.prec)
    path = save(res, args.out)
    print(json.dumps({"path": path, "prec": args.prec, "table": res["table"]}))


if __name__ == "__main__":
    main()
