"""The internal block-Schur interface of the general path: block normal equations filled on the
host and their damped Schur solve on the GB300.

Mirrors `plamatrix::internal::BlockNormalEquations<double>` and
`plamatrix::internal::solveDampedSchurComplement` as the reference uses them
(src/internal/BundleAdjustPlaMatrixAssembly.cpp:356-440, :843-912;
src/internal/BundleAdjustPlaMatrix.cpp:311-399; src/linescan_plamatrix.cpp:147-158), over the C ABI
of include/pb_gpu.h (`pb_bne_*`, `pb_gpu_solve_damped_schur`).  The container lives in host
memory; the elimination, the reduced solve and the back-substitution run on the device.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import native


class SchurSolveError(RuntimeError):
    """Raised for a breakdown; the message carries "numerically SPD" / "positive definite", which
    the reference's driver treats as a retryable linear failure (BundleAdjustPlaMatrix.cpp:34-40)."""


def _arr(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype)


class BlockNormalEquations:
    """BlockNormalEquations<double>(primaryBlocks, eliminatedBlocks, primaryBlockSize,
    eliminatedBlockSize): H x = -g with H_bc += w J_b^T J_c and g_b += w J_b^T r per residual."""

    def __init__(self, primary_blocks: int, eliminated_blocks: int, primary_block_size: int = 13,
                 eliminated_block_size: int = 3):
        self.L = native.load()
        self.h = C.c_void_p()
        st = self.L.pb_bne_create(primary_blocks, eliminated_blocks, primary_block_size, eliminated_block_size,
                                  C.byref(self.h))
        native.check(self.L, None, st, "pb_bne_create")
        self.primary_block_size = primary_block_size
        self.eliminated_block_size = eliminated_block_size

    def close(self):
        if self.h:
            self.L.pb_bne_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        native.check(self.L, None, st, what)

    def sizes(self):
        s = np.zeros(6, np.int32)
        self._check(self.L.pb_bne_sizes(self.h, s.ctypes.data), "pb_bne_sizes")
        keys = ("primaryBlockCount", "eliminatedBlockCount", "primaryBlockSize", "eliminatedBlockSize",
                "primaryPairs", "couplings")
        return {k: int(v) for k, v in zip(keys, s)}

    def clearValues(self):
        self._check(self.L.pb_bne_clear_values(self.h), "clearValues")

    def addResidualBlocks(self, primary, primary_jacobians, eliminated, eliminated_jacobian, residual, weight=1.0):
        r = _arr(residual)
        prim = _arr(primary, np.int32)
        jac = [_arr(j) for j in primary_jacobians]
        ptrs = (C.c_void_p * max(1, len(jac)))(*[j.ctypes.data for j in jac])
        je = None if eliminated is None or eliminated < 0 else _arr(eliminated_jacobian)
        self._check(self.L.pb_bne_add_residual_blocks(self.h, prim.ctypes.data if prim.size else None, ptrs,
                                                      len(jac), -1 if je is None else int(eliminated),
                                                      None if je is None else je.ctypes.data, r.ctypes.data,
                                                      r.size, float(weight)), "addResidualBlocks")

    def addPrimaryResidualBlocks(self, primary, primary_jacobians, residual, weight=1.0):
        self.addResidualBlocks(primary, primary_jacobians, -1, None, residual, weight)

    def addPrimaryResidualBlock(self, block, jacobian, residual, weight=1.0):
        self.addResidualBlocks([block], [jacobian], -1, None, residual, weight)

    def addEliminatedResidualBlock(self, block, jacobian, residual, weight=1.0):
        self.addResidualBlocks([], [], block, jacobian, residual, weight)

    def addPrimaryGradientBlock(self, block, gradient):
        g = _arr(gradient)
        self._check(self.L.pb_bne_add_primary_gradient_block(self.h, block, g.ctypes.data), "addPrimaryGradientBlock")

    def addPrimaryHessianBlock(self, row, col, block):
        b = _arr(block)
        self._check(self.L.pb_bne_add_primary_hessian_block(self.h, row, col, b.ctypes.data), "addPrimaryHessianBlock")

    def finalizePrimaryDiagonal(self, scale, add):
        self._check(self.L.pb_bne_finalize_primary_diagonal(self.h, scale, add), "finalizePrimaryDiagonal")

    def mergeFrom(self, other: "BlockNormalEquations"):
        self._check(self.L.pb_bne_merge_from(self.h, other.h), "mergeFrom")

    def mergeEliminatedShardFrom(self, shard: "BlockNormalEquations", offset: int):
        self._check(self.L.pb_bne_merge_eliminated_shard_from(self.h, shard.h, offset), "mergeEliminatedShardFrom")

    def export(self):
        """Dense primary matrix, primary gradient, eliminated blocks and gradient, couplings."""
        s = self.sizes()
        P, E, n, m, nc = (s["primaryBlockCount"], s["eliminatedBlockCount"], s["primaryBlockSize"],
                          s["eliminatedBlockSize"], s["couplings"])
        out = {"H": np.zeros((P * n, P * n)), "g": np.zeros(P * n), "Hee": np.zeros((E, m, m)), "ge": np.zeros((E, m)),
               "coupling_index": np.zeros((nc, 2), np.int32), "W": np.zeros((nc, n, m))}
        self._check(self.L.pb_bne_export(self.h, *(out[k].ctypes.data for k in
                                                   ("H", "g", "Hee", "ge", "coupling_index", "W"))), "export")
        return out


@dataclass
class SchurComplementSolverOptions:
    """SchurComplementSolverOptions as the reference fills them (BundleAdjustPlaMatrix.cpp:317-340)."""

    maxIterations: int = 0
    relativeTolerance: float = 1.0e-12
    absoluteTolerance: float = 1.0e-12
    preconditionerClusterSize: int = 1
    useInitialGuess: bool = False
    useMixedPrecision: bool = False


def solve_damped_schur_complement(ctx, equations: BlockNormalEquations, damping: float,
                                  options: SchurComplementSolverOptions = None, initial_guess=None):
    """solveDampedSchurComplement(equations, damping, options, workspace, &primary, &eliminated) on
    the context's GPU.  Returns (primary step, eliminated step, report dict); raises
    SchurSolveError on a breakdown."""
    o = options or SchurComplementSolverOptions()
    s = equations.sizes()
    x = np.zeros(s["primaryBlockCount"] * s["primaryBlockSize"])
    y = np.zeros(s["eliminatedBlockCount"] * s["eliminatedBlockSize"])
    if o.useInitialGuess:
        x[:] = _arr(initial_guess)
    co = native.SchurOptionsC(o.maxIterations, o.relativeTolerance, o.absoluteTolerance,
                              o.preconditionerClusterSize, int(o.useInitialGuess), int(o.useMixedPrecision))
    rep = native.SchurReportC()
    st = ctx.L.pb_gpu_solve_damped_schur(ctx.ctx, equations.h, float(damping), C.byref(co), x.ctypes.data,
                                         y.ctypes.data, C.byref(rep))
    if st == 4:  # PB_ERR_SINGULAR_BLOCK
        raise SchurSolveError(ctx.L.pb_gpu_last_error(ctx.ctx).decode())
    native.check(ctx.L, ctx.ctx, st, "solveDampedSchurComplement")
    return x, y, rep.as_dict()
