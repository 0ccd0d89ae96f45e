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

With ``host_io=True`` the step is driven from host memory, as an optimiser
on the host would drive it:
- the graph itself holds the copies: pinned host inputs → device at its
  start, and every output → pinned host memory at its end;
- a call copies the host inputs into the pinned staging, replays the graph
  once and waits for it;
- it returns the pinned host outputs (``None`` where the step returned
  ``None``), overwritten by the next call.
One graph launch per step replaces the separate copy launches around it.
"""

from __future__ import annotations

import torch

__all__ = ["GraphedStep"]


class GraphedStep:
    """``GraphedStep(fn, *example_inputs, host_io=False)`` -> callable replaying ``fn``
    as a CUDA graph (``host_io``: host inputs and outputs, copies inside the graph)."""

    def __init__(self, fn, *example_inputs, warmup: int = 3, host_io: bool = False):
        if not torch.cuda.is_available():
            raise RuntimeError("GraphedStep needs a CUDA device")
        self.fn = fn
        self.host_io = bool(host_io)
        self.static_in = [t.detach().to("cuda").clone() for t in example_inputs]
        self.stream = torch.cuda.Stream()
        self.stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(self.stream):
            for _ in range(max(1, warmup)):   # plan creation, allocator warm-up
                out = fn(*self.static_in)
        torch.cuda.current_stream().wait_stream(self.stream)
        torch.cuda.synchronize()
        if self.host_io:
            # pinned staging, allocated before capture
            self.host_in = [torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                            for t in self.static_in]
            for h, t in zip(self.host_in, self.static_in):
                h.copy_(t.cpu())
            self._single = not isinstance(out, (tuple, list))
            outs = (out,) if self._single else tuple(out)
            self.host_out = [None if o is None else
                             torch.empty(o.shape, dtype=o.dtype, pin_memory=True) for o in outs]
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            if self.host_io:
                for dst, h in zip(self.static_in, self.host_in):
                    dst.copy_(h, non_blocking=True)
            self.static_out = fn(*self.static_in)
            if self.host_io:
                outs = (self.static_out,) if self._single else tuple(self.static_out)
                if len(outs) != len(self.host_out):
                    raise RuntimeError("the step returned a different number of outputs "
                                       "during capture")
                for h, o in zip(self.host_out, outs):
                    if h is not None:
                        h.copy_(o, non_blocking=True)

    def __call__(self, *inputs):
        if len(inputs) != len(self.static_in):
            raise ValueError(f"expected {len(self.static_in)} inputs, got {len(inputs)}")
        for dst, src in zip(self.static_in, inputs):
            if dst.shape != src.shape:
                raise ValueError(f"input shape {tuple(src.shape)} != captured {tuple(dst.shape)}")
        if self.host_io:
            for h, src in zip(self.host_in, inputs):
                h.copy_(src)   # host -> pinned staging; the graph copies it to the device
            self.graph.replay()
            torch.cuda.current_stream().synchronize()
            return self.host_out[0] if self._single else tuple(self.host_out)
        for dst, src in zip(self.static_in, inputs):
            dst.copy_(src, non_blocking=True)
        self.graph.replay()
        return self.static_out
