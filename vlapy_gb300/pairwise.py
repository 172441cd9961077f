"""NumPy's pairwise summation tree, as a table the FP64 kernels replay.

``np.trapezoid(y, dx)`` (the reference's ``np.trapz``, e.g.
vlapy/core/field.py:36) forms ``t_j = (dx * (y[j+1] + y[j])) / 2`` and sums the
``n = len(y) - 1`` terms with NumPy's pairwise reduction: blocks of at most
128 terms are summed with eight interleaved accumulators, larger ranges are
split at ``n/2`` rounded down to a multiple of 8 and the halves added.  The
FP64 mode of the CUDA kernels evaluates the same tree so that densities and
moments agree with the reference bit for bit when f does; with ``1 - n``
cancelling in the Poisson solve, that is what keeps the field within 1e-12.

``leaf_program(n)`` returns the leaves (start, length) and a post-order
program: an entry ``k >= 0`` pushes leaf k's sum, ``-1`` pops two values and
pushes their sum (left + right).
"""

from __future__ import annotations

import numpy as np

BLOCK = 128
UNROLL = 8


def leaf_program(n: int):
    leaves: list[tuple[int, int]] = []
    prog: list[int] = []

    def rec(start: int, length: int):
        if length <= BLOCK:
            prog.append(len(leaves))
            leaves.append((start, length))
            return
        half = length // 2
        half -= half % UNROLL
        rec(start, half)
        rec(start + half, length - half)
        prog.append(-1)

    rec(0, n)
    return leaves, prog


def leaf_sum(a) -> float:
    """Sum of one leaf in NumPy's order (eight accumulators, then the tail)."""
    n = len(a)
    if n < UNROLL:
        r = 0.0
        for x in a:
            r += float(x)
        return r
    acc = [float(a[j]) for j in range(UNROLL)]
    i = UNROLL
    while i < n - (n % UNROLL):
        for j in range(UNROLL):
            acc[j] += float(a[i + j])
        i += UNROLL
    res = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]))
    while i < n:
        res += float(a[i])
        i += 1
    return res


def pairwise_sum(a) -> float:
    leaves, prog = leaf_program(len(a))
    stack: list[float] = []
    for op in prog:
        if op >= 0:
            s, ln = leaves[op]
            stack.append(leaf_sum(a[s:s + ln]))
        else:
            r = stack.pop()
            l = stack.pop()
            stack.append(l + r)
    return stack[0] if stack else 0.0


def trapz_emulated(y, dx) -> float:
    y = np.asarray(y, dtype=np.float64)
    t = (dx * (y[1:] + y[:-1])) / 2.0
    return pairwise_sum(t)


def device_table(n: int) -> np.ndarray:
    """Packed int32 table for the kernels: [n_leaves, n_prog, (start, len) *
    n_leaves, prog...]."""
    leaves, prog = leaf_program(n)
    out = [len(leaves), len(prog)]
    for s, ln in leaves:
        out += [s, ln]
    out += prog
    return np.asarray(out, dtype=np.int32)


def max_stack_depth(n: int) -> int:
    _, prog = leaf_program(n)
    d = m = 0
    for op in prog:
        d += 1 if op >= 0 else -1
        m = max(m, d)
    return m
