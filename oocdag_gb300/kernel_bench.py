"""Kernel-level micro-benchmarks (CUDA-event timing on the library's compute stream).

    python -m oocdag_gb300.kernel_bench syrk  --m 8192 --k 512 --prec bf16x3 [--reps 3]
    python -m oocdag_gb300.kernel_bench mixed --n 16384 --nb 256 --prec bf16x3 [--stored]
    python -m oocdag_gb300.kernel_bench batched --count 2000 --prec fp32 [--reps 2]

``syrk`` times one trailing-update launch C -= X X^T (lower, FP64 C) in the given
precision and prints the useful FP64-equivalent rate and the C read+write bandwidth;
``mixed`` times one mixed-precision factorization plus refinement of a seeded system
(generated in place, or with ``--stored`` a stored device matrix, which the library
factors over left-looking column blocks);
``batched`` times the persistent batched factor + solve of `count` seeded small systems.
These are the commands the profile summaries under profiles/ were captured with.
"""
from __future__ import annotations

import argparse
import json
import math


def _events(h):
    import torch

    s = torch.cuda.ExternalStream(h.stream(0))
    return s, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def syrk(args) -> None:
    import torch

    import oocdag_gb300 as ooc

    h = ooc.Handle(0)
    m, k = args.m, args.k
    X = torch.randn((k, m), dtype=torch.float64, device="cuda")  # column-major m x k
    C = torch.randn((m, m), dtype=torch.float64, device="cuda")
    for prec in args.prec:
        for rep in range(args.reps):
            s, e0, e1 = _events(h)
            torch.cuda.synchronize()
            e0.record(s)
            h.dsyrk_ln(prec, m, k, X, m, C, m)
            e1.record(s)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            print(json.dumps({"kernel": f"syrk_{prec}", "m": m, "k": k, "rep": rep, "ms": ms,
                              "useful_tflops": m * m * k / ms / 1e9,
                              "c_rmw_gbs": m * m / 2 * 16 / ms / 1e6}), flush=True)
    h.close()


def mixed(args) -> None:
    import torch

    import oocdag_gb300 as ooc

    h = ooc.Handle(0)
    if args.tail_order is not None:  # orders factored with nb/2-wide panels (0: uniform nb)
        h.set_option(ooc.OPT_TAIL_ORDER, args.tail_order)
    n, nb = args.n, args.nb
    alpha = 0.5774 * math.sqrt(n) * (1 + args.delta)
    B = torch.empty((1, n), dtype=torch.float64, device="cuda")
    X = torch.empty_like(B)
    h.gen_normal(B, n, n, 1, 7)
    A = None
    if args.stored:  # a stored device matrix: the library's left-looking block schedule applies
        if args.block_cols is not None:
            h.set_option(ooc.OPT_BLOCK_COLS, args.block_cols)
        A = torch.empty((n, n), dtype=torch.float64, device="cuda")
        h.matgen_uniform(A, n, n, 100, alpha)
    for prec in args.prec:
        for rep in range(args.reps):
            if A is not None:
                F = h.factor(A, n, n, nb, prec)
                it, be = F.refine(A, n, B, n, X, n, 1, 1e-14, 30)
            else:
                F = h.factor_gen(n, 100, alpha, nb, prec)
                it, be = F.refine_gen(B, n, X, n, 1, 1e-14, 30)
            print(json.dumps({"kind": "mixed", "prec": prec, "n": n, "nb": nb, "rep": rep,
                              "factor_s": F.stats["seconds"], "tflops": n ** 3 / 3 / F.stats["seconds"] / 1e12,
                              "iterations": it, "backward_error": be}), flush=True)
            F.close()
    h.close()


def batched(args) -> None:
    """`count` systems n ~ U{16..512} (numpy seed `seed`), A = M M^T / n + I, through the
    persistent batched kernel `reps` times with the given panel-width table."""
    import numpy as np

    import oocdag_gb300 as ooc
    from oocdag_gb300 import autotune

    h = ooc.Handle(0)
    rng = np.random.default_rng(args.seed)
    ns = [int(x) for x in rng.integers(16, 513, size=args.count)]
    A0, B0, a_off, b_off = autotune.make_batch(ns, 7, args.prec)
    flops = sum(n ** 3 / 3 for n in ns)
    for rep in range(args.reps):
        A, B = A0.clone(), B0.clone()
        info, sec = h.batched_posv(args.prec, ns, a_off, b_off, A, B, blk_table=args.table)
        if any(info):
            raise RuntimeError("a batched system failed")
        print(json.dumps({"kind": "batched", "prec": args.prec, "count": args.count, "rep": rep, "seconds": sec,
                          "tflops": flops / sec / 1e12}), flush=True)
    h.close()


def main() -> None:
    p = argparse.ArgumentParser()
    sub = p.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("syrk")
    a.add_argument("--m", type=int, default=8192)
    a.add_argument("--k", type=int, default=512)
    a.add_argument("--prec", nargs="+", default=["bf16x3"])
    a.add_argument("--reps", type=int, default=3)
    b = sub.add_parser("mixed")
    b.add_argument("--n", type=int, default=16384)
    b.add_argument("--nb", type=int, default=256)
    b.add_argument("--delta", type=float, default=0.1)
    b.add_argument("--prec", nargs="+", default=["bf16x3"])
    b.add_argument("--reps", type=int, default=1)
    b.add_argument("--tail-order", type=int, default=None,
                   help="OOC_OPT_TAIL_ORDER for the factor (default: the library's; 0: uniform nb-wide panels)")
    b.add_argument("--stored", action="store_true",
                   help="factor a stored device matrix (left-looking blocks) instead of generating it in place")
    b.add_argument("--block-cols", type=int, default=None, help="OOC_OPT_BLOCK_COLS with --stored")
    c = sub.add_parser("batched")
    c.add_argument("--count", type=int, default=2000)
    c.add_argument("--prec", default="fp32", choices=["fp64", "fp32"])
    c.add_argument("--seed", type=int, default=5)
    c.add_argument("--reps", type=int, default=2)
    c.add_argument("--table", type=int, nargs=16,
                   default=[64, 32, 32, 32, 32, 32, 32, 32, 64, 64, 64, 64, 64, 64, 64, 64])
    args = p.parse_args()
    {"syrk": syrk, "mixed": mixed, "batched": batched}[args.cmd](args)


if __name__ == "__main__":
    main()
