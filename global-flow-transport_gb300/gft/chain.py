"""Global-transport frame chain with checkpointed adjoint.

d_{t+1} = warp(d_t, v_t) (MacCormack + MC_SMOOTH) for t = 0..T-2, every frame
rendered by all views and compared with its targets (Sequence.densities_advect_fwd,
data_structures.py:1309-1320, plus the per-frame render loss of the
reconstruction loop).  The reference keeps every frame's grids and tape alive;
here only every k-th density is stored and each segment of k frames is
recomputed during the backward pass (torch.utils.checkpoint), so peak memory is
O(T/k + k) grids instead of O(T).
"""
import torch
from torch.utils.checkpoint import checkpoint

from . import fused, ops
from .pipeline import RenderAdvectStep


class TransportChain:
    def __init__(self, step: RenderAdvectStep, frames=16, checkpoint_every=4):
        self.step = step
        self.T = frames
        self.k = max(1, checkpoint_every)

    def _segment(self, d, vels, targets, t0, t1):
        """Frames t0..t1-1 starting from density d at frame t0; returns the
        density at frame t1 (or the last one) and the segment's loss."""
        s = self.step
        loss = d.new_zeros(())
        for t in range(t0, t1):
            img = s.render(d)
            if s.mode == 'plain':
                rgb = img[..., :3] + s.bkg * torch.exp(-img[..., 3:])
                loss = loss + torch.mean((rgb - targets[t]) ** 2)
            else:
                loss = loss + fused.image_loss(img, targets[t], s.bkg_host, getattr(s, "tonemap", "NONE"))
            if t + 1 < self.T:
                vx, vy, vz = vels[t]
                d = s.advect(d, vx, vy, vz)
        return d, loss

    def loss(self, d0, vels, targets, use_checkpoints=True):
        d = d0
        total = d0.new_zeros(())
        for t0 in range(0, self.T, self.k):
            t1 = min(self.T, t0 + self.k)
            if use_checkpoints:
                d, l = checkpoint(self._checkpointed, d, vels, targets, t0, t1, use_reentrant=False,
                                  preserve_rng_state=False)  # no randomness; capturable
            else:
                d, l = self._segment(d, vels, targets, t0, t1)
            total = total + l
        return total

    def _checkpointed(self, d, vels, targets, t0, t1):
        # A checkpointed segment's backward runs on the nodes of its first
        # forward and only regenerates their saved tensors by running the
        # segment again; the contexts of that second run are dropped.  So
        # neither run may start a raymarch gradient's weight pass ahead on a
        # side stream: the passes run in the backward.
        with ops.side_stream_weights(False):
            return self._segment(d, vels, targets, t0, t1)
