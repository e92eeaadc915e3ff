"""simwave_gb300: simwave's forward time-stepping operator on GB300 (sm_103a).

Same public API as simwave (simwave/__init__.py:1-41) for the propagation
path: ``SpaceModel``, ``TimeModel``, ``Source``, ``Receiver``, ``Wavelet``,
``RickerWavelet``, ``MultiWavelet``, ``Solver`` and ``Compiler``, where
``Compiler(language='cuda_sm100a')`` (the default) selects the GPU library.
"""
from .backend.compiler import Compiler
from .frontend.model import SpaceModel, TimeModel
from .frontend.solver import Solver
from .frontend.source import (MultiWavelet, Receiver, RickerWavelet, Source,
                              Wavelet)

__all__ = ["Compiler", "SpaceModel", "TimeModel", "Source", "Receiver",
           "Wavelet", "RickerWavelet", "MultiWavelet", "Solver"]
