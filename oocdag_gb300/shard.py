"""Several GPUs on one matrix: the layout and exchange schedule of the tiled factorization.

The target machine has several GPUs per node, but every call that runs this library's GPU
code here gets exactly one GPU, so the multi-GPU factorization is carried as a host-side
schedule that CPU ranks execute (torch.distributed, gloo), with the tile arithmetic of the
reference's task bodies: dpotrf on the diagonal tile (oocquark.cpp:87), dtrsm R/L/T/N below
it (:130), dsyrk/dgemm updates of later columns (:176, :222).  It is the schedule a GPU
rank would follow with the library's kernels in place of those bodies; that GPU path is not
built, since nothing here could run or measure it.

Layout: tile columns are dealt block-cyclically, column k to rank k % world; a rank keeps
the full height (rows k*nb .. n-1) of each column it owns, as a GPU would keep them in its
own HBM.  Schedule, for every tile column k in order:

  1. the owner factors the diagonal tile and solves the tiles below it (the column is
     final: every earlier column's update was applied on receipt);
  2. the finished column is broadcast to every rank (host-staged, or a collective into
     each GPU's own memory; no rank reads another's memory);
  3. every rank applies it to the later columns it owns.

One broadcast per tile column is the only exchange; its bytes are the lower triangle once
per rank that receives it.  `bench.py --gpus N` does not use this (it runs N independent
replicas, one matrix per GPU).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def owner(k: int, world: int) -> int:
    """Rank that owns tile column k."""
    return k % world


@dataclass
class Plan:
    n: int
    nb: int
    world: int
    columns: list[list[int]]      # tile columns owned by each rank
    broadcast_bytes: int          # FP64 bytes each broadcast moves, summed over columns


def plan(n: int, nb: int, world: int) -> Plan:
    if n <= 0 or nb <= 0 or world <= 0:
        raise ValueError("n, nb and world must be positive")
    bb = (n + nb - 1) // nb
    cols = [[k for k in range(bb) if owner(k, world) == r] for r in range(world)]
    total = 0
    for k in range(bb):
        rows = n - k * nb
        total += rows * min(nb, n - k * nb) * 8
    return Plan(n, nb, world, cols, total)


def _chol_lower(a: np.ndarray) -> np.ndarray:
    import scipy.linalg as sla

    return sla.cholesky(a, lower=True, check_finite=False)


def factor(A: np.ndarray, nb: int, group=None) -> tuple[dict[int, np.ndarray], int]:
    """Factor the SPD matrix A (every rank passes the same A; each keeps only its columns).

    Returns ({tile column k: its final rows k*nb.. of L, for the columns this rank owns},
    info) with LAPACK info (0, or the order of the first non-positive leading minor).
    """
    import scipy.linalg as sla
    import torch
    import torch.distributed as dist

    n = A.shape[0]
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    bb = (n + nb - 1) // nb
    mine = {k: np.array(A[k * nb:, k * nb:k * nb + min(nb, n - k * nb)], dtype=np.float64, order="F")
            for k in range(bb) if owner(k, world) == rank}
    info = 0
    for k in range(bb):
        k0, w = k * nb, min(nb, n - k * nb)
        src = owner(k, world)
        buf = torch.empty((n - k0) * w + 1, dtype=torch.float64)
        if rank == src:
            col = mine[k]
            if info == 0:
                try:
                    col[:w, :] = _chol_lower(col[:w, :])
                    if n - k0 > w:
                        col[w:, :] = sla.solve_triangular(col[:w, :], col[w:, :].T, lower=True,
                                                          check_finite=False).T
                except np.linalg.LinAlgError:
                    # LAPACK info: first column of this tile whose pivot is not positive
                    d = col[:w, :].copy()
                    j = 0
                    while j < w:
                        if d[j, j] <= 0:
                            break
                        d[j, j] = np.sqrt(d[j, j])
                        d[j + 1:, j] /= d[j, j]
                        d[j + 1:, j + 1:] -= np.outer(d[j + 1:, j], d[j + 1:, j])
                        j += 1
                    info = k0 + j + 1
            buf[:-1] = torch.from_numpy(np.ascontiguousarray(col.reshape(-1, order="F")))
            buf[-1] = float(info)
        if world > 1:
            dist.broadcast(buf, src=src, group=group)
        info = int(buf[-1].item())
        if info:
            break
        Lk = buf[:-1].numpy().reshape((n - k0, w), order="F")
        for c, col in mine.items():
            if c <= k:
                continue
            c0 = c * nb
            # rows c0.. of column c -= L(c0.., k) L(c block, k)^T
            col -= Lk[c0 - k0:, :] @ Lk[c0 - k0:c0 - k0 + col.shape[1], :].T
    return mine, info


def assemble(parts: dict[int, np.ndarray], n: int, nb: int) -> np.ndarray:
    """Lower triangle of L from the columns one rank owns (zeros elsewhere)."""
    L = np.zeros((n, n))
    for k, col in parts.items():
        k0 = k * nb
        L[k0:, k0:k0 + col.shape[1]] = col
    return np.tril(L)
