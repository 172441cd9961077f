"""Fokker-Planck operator names (mirror of the selection logic of
vlapy/core/collisions.py:268-317).  The diagonals and the tridiagonal solve
run fused on the device (libvlagpu vg_collision_step): the Lenard-Bernstein
("lb", :26-83) and Dougherty ("dg", :86-160) matrices are built per x row
from FP64 trapz moments and solved by the Thomas recurrence of :222-265."""

from __future__ import annotations

OPERATORS = ("lb", "dg")
SOLVERS = ("batched_tridiagonal", "naive")


def check_names(fokker_planck: dict):
    op = fokker_planck.get("type")
    solver = fokker_planck.get("solver", "batched_tridiagonal")
    if op not in OPERATORS:
        raise NotImplementedError("Collision Operator: <" + str(op) + "> has not yet been implemented")
    if solver not in SOLVERS:
        raise NotImplementedError("Matrix Solver: <" + str(solver) + "> has not yet been implemented")
    return op, solver
