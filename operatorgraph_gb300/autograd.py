"""torch.autograd binding of the derivation and its adjoint.

`derive_transforms(engine, axioms, blocks, sizes)` derives the batch with the
per-axiom parameter blocks `blocks` (flat float32, numBlocks x blockStride)
and axiom sizes `sizes` (numAxioms x 3) and returns the terminal transforms
M (n x 12, row-major 3x4) and their derivation-path hashes (int64, for
matching terminals between runs; the emission order is free).  Backward runs
pga_adjoint on the engine's recorded tape: the discrete derivation (branches,
repetition counts, discards) is the one of this forward pass.

The engine must be created with record_tape=True, and backward must run before
the engine derives again (the tape holds one derivation).

`PathTarget` holds a target derivation's terminal centres and extents keyed
by derivation path, and `PathTarget.sse(M, paths)` is the fitting loss of
differentiable facade fitting: the sum of squared errors of the centres
(M[:, 3, 7, 11]) and the extents (the lengths of M's first three columns,
the terminal's size along its own axes) over terminals matched by path.
"""
import numpy as np
import torch

from . import grammar as G

_SIZE = slice(4, 7)  # PgaAxiom.size as float32 words


class _Derive(torch.autograd.Function):
    @staticmethod
    def forward(ctx, blocks, sizes, engine, axioms, capacity):
        d_ax = axioms.clone()
        n_ax = d_ax.numel() // G.AXIOM_DT.itemsize
        d_ax.view(torch.float32).view(n_ax, 12)[:, _SIZE] = sizes.detach().to(torch.float32)
        blk = blocks.detach().contiguous().to(torch.float32) if blocks is not None else None
        out, n, _ = engine.execute(d_ax, blocks=blk, capacity=capacity)
        rec = out[:n]
        M = rec.view(torch.float32).view(n, 16)[:, :12].clone()
        paths = rec.view(torch.int64).view(n, 8)[:, 7].clone()
        ctx.engine = engine
        ctx.num_blocks = 0 if blocks is None else blocks.numel() // max(engine.block_stride, 1)
        ctx.num_axioms = n_ax
        ctx.has_blocks = blocks is not None
        ctx.keep = (d_ax, blk)  # device inputs the tape refers to
        ctx.mark_non_differentiable(paths)
        return M, paths

    @staticmethod
    def backward(ctx, gM, gPaths):
        eng = ctx.engine
        gM = gM.contiguous().to(torch.float32)
        g_blocks = torch.zeros(max(ctx.num_blocks * eng.block_stride, 1), dtype=torch.float32, device=gM.device)
        g_sizes = torch.zeros((ctx.num_axioms, 3), dtype=torch.float32, device=gM.device)
        eng.adjoint_raw(gM.data_ptr(), g_blocks.data_ptr() if ctx.has_blocks else None, ctx.num_blocks,
                        g_sizes.data_ptr())
        return (g_blocks[: ctx.num_blocks * eng.block_stride] if ctx.has_blocks else None), g_sizes, None, None, None


def axioms_tensor(axioms, device="cuda"):
    return torch.from_numpy(np.ascontiguousarray(axioms).view(np.uint8).reshape(-1).copy()).to(device)


def derive_transforms(engine, axioms, blocks, sizes, capacity):
    """Differentiable derivation: (M [n, 12], paths [n]) from blocks and axiom sizes."""
    return _Derive.apply(blocks, sizes, engine, axioms, capacity)


def centres_extents(M):
    """Terminal centres (n x 3) and extents (n x 3, the column lengths of the
    3 x 3 part of model * scale(size)) of transforms M (n x 12)."""
    c = M[:, [3, 7, 11]]
    R = M.reshape(-1, 3, 4)[:, :, :3]
    return c, torch.sqrt((R * R).sum(dim=1))


class PathTarget:
    """Centres and extents of a target derivation, keyed by derivation path."""

    def __init__(self, M, paths):
        order = torch.argsort(paths)
        self.paths = paths[order]
        self.c, self.e = centres_extents(M.detach()[order])

    def sse(self, M, paths, check=True):
        """Sum of squared errors of centres and extents against the target;
        check=True verifies that the derivation has exactly the target's
        paths (no branch, repetition count or discard changed)."""
        order = torch.argsort(paths)
        if check and not torch.equal(paths[order], self.paths):
            raise ValueError("the derivation's paths differ from the target's")
        c, e = centres_extents(M[order])
        return ((c - self.c) ** 2).sum() + ((e - self.e) ** 2).sum()
