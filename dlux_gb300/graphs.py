"""Replay a whole PSF (+ gradient) step as one CUDA graph.

A small problem, such as a 256² pupil at one wavelength, spends most of its
step on the host: Python dispatch of the layer objects, autograd and a few
dozen launches. The device work is a fraction of a millisecond. A graph
captures the step once: the forward kernels, the hand-written reverse kernels
reached through autograd, and the torch glue. Each later call is then one
graph launch.

The step function takes and returns tensors. Its inputs are copied into
static device buffers before each replay. Its outputs are the captured
output tensors, overwritten by every replay: copy them out if they must
survive the next call. The function must not synchronise the host or depend
on host values that change between calls; anything that differs per call has
to be an input tensor. Every library call on the step's path allocates from
stream-ordered pools or preallocated plan buffers, which keeps the step
capturable. The first calls, made before capture, create the plans.
"""

from __future__ import annotations

import torch

__all__ = ["GraphedStep"]


class GraphedStep:
    """``GraphedStep(fn, *example_inputs)`` -> callable replaying ``fn`` as a CUDA graph."""

    def __init__(self, fn, *example_inputs, warmup: int = 3):
        if not torch.cuda.is_available():
            raise RuntimeError("GraphedStep needs a CUDA device")
        self.fn = fn
        self.static_in = [t.detach().clone() for t in example_inputs]
        self.stream = torch.cuda.Stream()
        self.stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(self.stream):
            for _ in range(max(1, warmup)):   # plan creation, allocator warm-up
                fn(*self.static_in)
        torch.cuda.current_stream().wait_stream(self.stream)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            self.static_out = fn(*self.static_in)

    def __call__(self, *inputs):
        if len(inputs) != len(self.static_in):
            raise ValueError(f"expected {len(self.static_in)} inputs, got {len(inputs)}")
        for dst, src in zip(self.static_in, inputs):
            if dst.shape != src.shape:
                raise ValueError(f"input shape {tuple(src.shape)} != captured {tuple(dst.shape)}")
            dst.copy_(src, non_blocking=True)
        self.graph.replay()
        return self.static_out
