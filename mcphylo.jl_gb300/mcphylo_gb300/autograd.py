"""The likelihood as a differentiable PyTorch operation of the branch lengths.

`phylo_loglik(engine, blen)` returns the per-instance log-likelihoods for the packed
branch lengths `blen` (a float64 CUDA tensor, instance after instance, num order, as
Engine.grad_offsets lays them out).  Its backward pass is the engine's pre-order
adjoint gradient (the gradlogpdf of Phylodist.jl:124-138), so samplers and
optimisers written in PyTorch can use the engine as an autograd node.  Inputs and
outputs stay on the device: the engine reads the branch lengths and writes logL and
the gradient in device memory, on PyTorch's current stream.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import Engine


class _PhyloLogLik(torch.autograd.Function):
    @staticmethod
    def forward(ctx, blen: torch.Tensor, engine: Engine):
        if not blen.is_cuda or blen.dtype != torch.float64 or blen.dim() != 1:
            raise ValueError("blen must be a 1-D float64 CUDA tensor")
        off = engine.grad_offsets()
        if blen.numel() != int(off[-1]):
            raise ValueError(f"blen has {blen.numel()} entries, the engine's trees have "
                             f"{int(off[-1])} branches")
        blen = blen.contiguous()
        ll = torch.empty(engine.M, dtype=torch.float64, device=blen.device)
        grad = torch.empty(int(off[-1]), dtype=torch.float64, device=blen.device)
        stream = torch.cuda.current_stream(blen.device)
        engine.set_stream(stream.cuda_stream)
        engine.set_all_branch_lengths_device(blen.data_ptr())
        engine.logpdf_grad_device(ll.data_ptr(), grad.data_ptr())
        if stream.cuda_stream == 0:
            # the legacy default stream does not order the engine's own stream
            engine.synchronize()
        counts = torch.as_tensor(np.diff(off), device=blen.device)
        ctx.save_for_backward(grad, counts)
        return ll

    @staticmethod
    def backward(ctx, grad_ll: torch.Tensor):
        grad, counts = ctx.saved_tensors
        return grad * torch.repeat_interleave(grad_ll, counts), None


def phylo_loglik(engine: Engine, blen: torch.Tensor) -> torch.Tensor:
    """Per-instance log-likelihoods (shape [M]) of the engine's trees at `blen`,
    differentiable with respect to `blen`."""
    return _PhyloLogLik.apply(blen, engine)
