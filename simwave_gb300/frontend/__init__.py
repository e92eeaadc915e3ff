"""Problem description: grids, time axis, sources/receivers, wavelets."""
from .model import SpaceModel, TimeModel
from .source import Source, Receiver, Wavelet, RickerWavelet, MultiWavelet

__all__ = ["SpaceModel", "TimeModel", "Source", "Receiver", "Wavelet",
           "RickerWavelet", "MultiWavelet"]
