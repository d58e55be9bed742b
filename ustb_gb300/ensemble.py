"""High-frame-rate ensembles: many frames of one acquisition per launch, replayed
from a CUDA graph.

An ensemble is F frames of int16 I/Q scanner samples recorded with the same
probe, scan and transmit sequence (e.g. 200 frames x 11 plane waves for Doppler
or functional imaging).  ``Ensemble`` keeps everything such a stream needs
resident on the device: the int16 input buffer, its FP16/BF16 storage copy, the
FP32 interpolation-entry workspace, the queue scratch and the output frames.
One ensemble costs one conversion kernel, one entry pass and ONE persistent
launch whose CTAs pull (frame, tile) work items from a queue; the three are
recorded once into a CUDA graph and replayed for every ensemble, so the host
issues one graph launch per ensemble.

The reference beamforms such data one ``midprocess.das`` call at a time, all
frames of a call through ``das_c``'s per-pixel loop (+midprocess/das.m:77-317,
+mex/source/das_c.cpp:355-409); ``das_cuda`` pipelines frames over two streams
(+mex/source/das_cuda.cu:253-283).
"""
from __future__ import annotations

from typing import Dict, Optional

import torch

from . import _lib, fast
from .enums import Dimension, Precision

SRC_INT16 = 1  # USTB_SRC_INT16


class Ensemble:
    """Beamform ensembles of ``F`` frames with one persistent launch per ensemble.

    ``geom``: the acquisition's ``fast.FastGeometry``; ``L``: samples per trace;
    ``scale``: factor from int16 counts to channel-data units (applied in the
    conversion).  Feed an ensemble with ``run(x)`` where ``x`` is an int16 tensor
    (host or device) of shape (F, W, N, L, 2): the ABI layout with I, Q last."""

    def __init__(self, geom: fast.FastGeometry, F: int, L: int, dimension=Dimension.both,
                 precision: Precision = Precision.fp16, scale: float = 1.0, graph: bool = True):
        self.geom, self.F, self.L = geom, int(F), int(L)
        self.precision, self.scale = Precision(precision), float(scale)
        self.dimension = int(dimension)
        dev = geom.device
        self.device = dev
        shape = (self.F, geom.W, geom.N, self.L, 2)
        self.input = torch.zeros(shape, dtype=torch.int16, device=dev)
        self.storage = torch.empty(shape, dtype=fast.TORCH_STORE[self.precision], device=dev)
        self.request = fast.Request(self.storage, self.precision, True, geom, self.dimension, F=self.F, L=self.L)
        self.workspace = torch.empty(max(fast.workspace_bytes([self.request]), 1), dtype=torch.uint8, device=dev)
        self.scratch = torch.zeros(2, dtype=torch.int64, device=dev)
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self.use_graph = bool(graph)

    @property
    def outputs(self) -> Dict[str, torch.Tensor]:
        """'cube': (F, Wk, Nk, P) complex64 frames in the ABI layout (filled by ``run``)."""
        return self.request.outputs

    def _launch(self) -> None:
        """Conversion + entries + persistent launch on the current stream."""
        st = torch.cuda.current_stream(self.device)
        with torch.cuda.device(self.device):
            _lib.call("ustb_convert_channels", self.input.data_ptr(), SRC_INT16, self.storage.data_ptr(),
                      fast.STORE[self.precision], self.input.numel(), self.scale, st.cuda_stream)
        fast.das_fast_batch([self.request], scratch=self.scratch, workspace=self.workspace)

    def capture(self) -> None:
        """Record the ensemble's work into a CUDA graph (after one eager run that sets
        up the kernels' attributes)."""
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self._launch()
        torch.cuda.current_stream(self.device).wait_stream(side)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            self._launch()
        self.graph = g

    def run(self, ensemble: Optional[torch.Tensor] = None) -> Dict[str, torch.Tensor]:
        """Beamform one ensemble (stream-ordered; read ``flags()`` or synchronise before
        using the outputs).  ``ensemble`` is copied into the resident input buffer
        first; None re-beamforms what the buffer holds."""
        if ensemble is not None:
            if tuple(ensemble.shape) != tuple(self.input.shape) or ensemble.dtype != torch.int16:
                raise ValueError(f"ensemble must be int16 {tuple(self.input.shape)}, got "
                                 f"{ensemble.dtype} {tuple(ensemble.shape)}")
            self.input.copy_(ensemble, non_blocking=True)
        if self.use_graph:
            if self.graph is None:
                self.capture()
            self.graph.replay()
        else:
            self._launch()
        return self.outputs

    def flags(self) -> int:
        """USTB_FLAG_* bits of the last run (synchronises)."""
        return int(self.scratch[0].item()) & 0xFFFFFFFF
